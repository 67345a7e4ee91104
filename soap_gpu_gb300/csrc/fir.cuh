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
FirPlanSizes fir_plan_sizes(int form, int n, int n_mu, long long gm, bool phase, int n_lists);

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
};
enum { FIR_STAGE_GEOMETRY = 1, FIR_STAGE_CUBES = 2, FIR_STAGE_RUN = 4 };

int fir_phase(soapgb_ctx *ctx, int form, const FirPhaseArgs &a, char *scratch, const FirPlanSizes &plan);
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
