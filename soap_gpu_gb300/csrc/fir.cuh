// Collapsed shift-FIR engine (FAST64 / FAST32 forms of the disk and phase integration).
#pragma once
#include "internal.cuh"

struct RegionPhase;

struct FirPlanSizes {
    size_t bytes = 0;
};

// workspace of the FAST forms: per-cell geometry for the G*G grid, the velocity order
// of the cells, per-list cell lists / prefix sums / segments and typed cube copies
// (one cube for the quiet disk, six for the phase integration)
// typed_external: the phase integration reads typed cubes shared with other stars
// (fir_typed_cubes), so the workspace holds none
FirPlanSizes fir_plan_sizes(int form, int n, int n_mu, long long gm, bool phase, int n_lists,
                            bool typed_external = false);

// typed copies of the seed cubes read by the phase integration (c[0], c[1]: the spot and
// facula classes' rows interleaved per pixel), shareable by the stars of a batch (they
// share the seed spectra)
struct FirTyped {
    const void *c[6];
    const double *spot_sed, *fac_sed;
    const void *spot_sed2, *fac_sed2;
};
size_t fir_typed_bytes(int form, int n, int n_mu);
// the addresses fir_typed_cubes writes at dst (no device work)
void fir_typed_layout(int form, int n, int n_mu, char *dst, const soapgb_cubes &c, FirTyped *out);
int fir_typed_cubes(soapgb_ctx *ctx, int form, int n, const soapgb_cubes &c, char *dst, FirTyped *out);

struct FirQuietArgs {
    int n, n_eff;
    const double *wave;
    const double *cube;     // n_mu x n (FP64, device)
    int n_mu;
    long long gm;           // G*G
    const double *delta, *limb;
    const int *region;
    double step;
    double *out;            // n (tail set to 0)
    double lambda0 = 0.0;   // wave[0] when known on the host (0: read from the device)
    // optional second cube of the same disk (its cell order, lists and sums shared)
    const double *cube2 = nullptr;
    double *out2 = nullptr;
};

int fir_quiet(soapgb_ctx *ctx, int form, const FirQuietArgs &a, char *scratch, const FirPlanSizes &plan);

struct FirPhaseArgs {
    int n, n_eff;
    const double *wave;
    const soapgb_cubes *cubes;  // device pointers, FP64
    int n_phase;
    const double *temp = nullptr, *bi = nullptr;   // n_phase x G*G maps, or null with `table`
    // without maps: the region table of the phases (regions.cuh); the lists are built
    // from the regions' bounding boxes (grids of at most fir_box_lists_max_gm() cells)
    const RegionPhase *table = nullptr;
    const int *reg_off = nullptr;   // n_phase + 1 (device)
    int grid = 0;
    int box_cap = 0;                // > 0: each phase sorts its active cells (capacity, from the boxes)
    // optional: the phases with a visible region (run) and the others (zero), ascending,
    // on the device and the host; the run stage then integrates only the former and
    // zero-fills the outputs of the latter (no active cell, so zero deficits)
    const int *run_list = nullptr, *zero_list = nullptr;
    const int *run_host = nullptr, *zero_host = nullptr;
    int n_run = 0, n_zero = 0;
    // 0: the zero phases' outputs are left unwritten (their consumer knows them as zero)
    int zero_fill = 1;
    const double *delta, *limb, *lb;
    const int *region;
    long long gm;               // G*G
    double step;
    const soapgb_activity *act;
    void *flux, *bconv, *tot;   // n_phase x n: float (FAST32) or double (FAST64)
    int out_f32;
    long long out_stride;       // distance between phases in the outputs
    // staged use (a pipeline that overlaps chunks of phases with their copies):
    // FIR_STAGE_GEOMETRY builds the cell order, lists and tile plans of all phases,
    // FIR_STAGE_CUBES the typed cube copies, FIR_STAGE_RUN integrates phases [l0, l1)
    int stage = 7;
    int l0 = 0, l1 = -1;        // l1 < 0: all phases
    double lambda0 = 0.0;       // wave[0] when known on the host (0: read from the device)
    const FirTyped *typed = nullptr;   // shared typed cubes (the workspace then has no cube slots)
};
enum { FIR_STAGE_GEOMETRY = 1, FIR_STAGE_CUBES = 2, FIR_STAGE_RUN = 4 };

int fir_phase(soapgb_ctx *ctx, int form, const FirPhaseArgs &a, char *scratch, const FirPlanSizes &plan);

// Several stars' phase integrations in one persistent launch (FP32 form).  Each star has
// run its geometry stage (fir_phase with FIR_STAGE_GEOMETRY and run lists) in its own
// workspace, with shared typed cubes; fir_phase_star_args writes its kernel arguments
// (fir_tile_args_bytes() bytes) to out, host memory.  fir_phase_multi then integrates
// the items (star, phase) of d_items (device, n_items) from the device copy of those
// arguments (d_star_args, one record per star); star0_args is a host copy of the first
// (its grid-wide fields).  chunk: positions per round-robin chunk (0: contiguous shares);
// blocks_per_sm: 0 for as many as fit.
size_t fir_tile_args_bytes();
int fir_phase_star_args(soapgb_ctx *ctx, int form, const FirPhaseArgs &a, char *scratch, void *out);
int fir_phase_multi(soapgb_ctx *ctx, int form, const void *star0_args, const void *d_star_args, const int2 *d_items,
                    int n_items, int chunk, int blocks_per_sm);
// largest G*G whose phase lists can be built from the region boxes
long long fir_box_lists_max_gm();
// capacity of the per-phase sort for phases of at most max_box_cells box cells (0: too many)
int fir_sorted_box_capacity(long long max_box_cells);

namespace soapgb {
// radix sorts of (key, cell) pairs on the context's stream (fir_sort.cu)
size_t fir_sort_temp_bytes(long long gm);
int fir_sort_u64(soapgb_ctx *ctx, long long gm, const unsigned long long *keys_in, unsigned long long *keys_out,
                 const int *vals_in, int *vals_out, void *temp, size_t temp_bytes);
int fir_sort_u32(soapgb_ctx *ctx, long long gm, const unsigned *keys_in, unsigned *keys_out, const int *vals_in,
                 int *vals_out, int end_bit, void *temp, size_t temp_bytes);
}  // namespace soapgb
