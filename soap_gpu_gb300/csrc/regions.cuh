// Per-(phase, region) constants of the active-region maps and the per-cell test that
// turns them into a cell's temperature and type (regions.cu; the collapsed integration
// builds its per-phase cell lists from the same test in fir.cu).
#pragma once
#include <vector>

#include "internal.cuh"

struct RegionPhase {
    int iy0, iz0, iy1, iz1;  // bounding box [iy0, iy1) x [iz0, iz1), clamped to the grid
    int visible;
    int type;                // 0 spot, 1 facula
    double s;                // cap chord radius
    double r0, r1, r2;       // first row of the inverse rotation
    float f0, f1, f2, fcap;  // FP32 copies of r0, r1, r2 and of 1 - s^2 (the FP32 owner test)
};

// Temperature t and type b of cell (iy, iz) after the regions [r0, r1) of one phase,
// applied in order (a later region overwrites an earlier one; -9999 outside every
// region), and the index of the region that set them (-1 if none).  One rounding per
// operation, as spot_scan (SOAP_integration.cu:326-390) evaluates it.
__device__ __forceinline__ int region_cell_value(const RegionPhase *__restrict__ table, int r0, int r1, int iy, int iz,
                                                 double delta_grid, int t_star, int t_diff_spot, int t_diff_fac,
                                                 double &t, double &b) {
    double y = 0.0, z = 0.0;
    bool have_yz = false;   // FP64 only for cells inside a bounding box
    int owner = -1;
    t = -9999.0;
    b = -9999.0;
    for (int r = r0; r < r1; ++r) {
        const RegionPhase rp = table[r];
        if (!rp.visible || iy < rp.iy0 || iy >= rp.iy1 || iz < rp.iz0 || iz >= rp.iz1) continue;
        if (!have_yz) {
            y = __dadd_rn(-1., __dmul_rn((double)iy, delta_grid));
            z = __dadd_rn(-1., __dmul_rn((double)iz, delta_grid));
            have_yz = true;
        }
        if (!(__dadd_rn(__dmul_rn(z, z), __dmul_rn(y, y)) < 1.)) continue;
        const double xa0 = __dsqrt_rn(__dsub_rn(1., __dadd_rn(__dmul_rn(y, y), __dmul_rn(z, z))));
        const double xi0 = __dadd_rn(__dadd_rn(__dmul_rn(rp.r0, xa0), __dmul_rn(rp.r1, y)), __dmul_rn(rp.r2, z));
        if (__dmul_rn(xi0, xi0) >= __dsub_rn(1., __dmul_rn(rp.s, rp.s))) {
            if (rp.type == 0) {
                t = (double)(t_star - t_diff_spot);
                b = 0.0;
            } else {
                const double tp = __dadd_rn(
                    __dsub_rn(__dadd_rn((double)(t_star + t_diff_fac), 0.9), __dmul_rn(407.7, xa0)),
                    __dmul_rn(190.9, __dmul_rn(xa0, xa0)));
                t = (double)(int)tp;
                b = 1.0;
            }
            owner = r;
        }
    }
    return owner;
}

// The index of the region that sets cell (iy, iz) -- the same answer as
// region_cell_value -- from FP32 arithmetic where that answer is certain, or -2 when
// a test lies within the FP32 error bound of its threshold (the caller then evaluates
// region_cell_value in FP64).  Error bound: y and z differ from the FP64 values by at
// most 3e-7, y^2 + z^2 by 1.6e-6; with 1 - y^2 - z^2 >= 1e-2 the square root differs
// by 2.1e-5, xi0 by 2.3e-5 and xi0^2 - (1 - s^2) by 4.7e-5.  The margins below are 10x
// (disk) and 4x (cap) those bounds; cells within 1e-2 of the limb go to FP64.
__device__ __forceinline__ int region_owner_fp32(const RegionPhase *__restrict__ table, int r0, int r1, int iy, int iz,
                                                 float delta_grid) {
    const float y = fmaf((float)iy, delta_grid, -1.f), z = fmaf((float)iz, delta_grid, -1.f);
    const float q = fmaf(y, y, z * z);
    int owner = -1;
    bool inside_disk = false, disk_known = false;
    for (int r = r0; r < r1; ++r) {
        const RegionPhase rp = table[r];
        if (!rp.visible || iy < rp.iy0 || iy >= rp.iy1 || iz < rp.iz0 || iz >= rp.iz1) continue;
        if (!disk_known) {
            if (fabsf(q - 1.f) <= 4e-5f) return -2;
            inside_disk = q < 1.f;
            disk_known = true;
        }
        if (!inside_disk) continue;
        const float rest = 1.f - q;
        if (rest < 1e-2f) return -2;
        const float xa = sqrtf(rest);
        const float xi = fmaf(rp.f0, xa, fmaf(rp.f1, y, rp.f2 * z));
        const float d = fmaf(xi, xi, -rp.fcap);
        if (fabsf(d) <= 2e-4f) return -2;
        if (d > 0.f) owner = r;
    }
    return owner;
}

namespace soapgb {
// The region table of n_phase phases built on the host and copied to scratch:
// *d_table (reg_off[n_phase] rows) and *d_off (n_phase + 1 offsets); phase_visible
// (optional) gets 1 for the phases with at least one visible region, else 0;
// max_box_cells (optional) the largest sum over a phase's visible regions of their
// bounding-box cells (a bound on the phase's active cells).  With `pack` the copies are
// not issued: *pack receives the image of the scratch bytes, for the caller to copy
// (with its own small uploads) in one go.
int phase_table_device(soapgb_ctx *ctx, int grid, double incl, int n_phase, const double *h_phases,
                       const int *h_reg_off, const double *h_regions, const soapgb_activity *act, char *scratch,
                       size_t scratch_bytes, const RegionPhase **d_table, const int **d_off,
                       std::vector<unsigned char> *phase_visible = nullptr, long long *max_box_cells = nullptr,
                       std::vector<char> *pack = nullptr);
size_t phase_maps_scratch_bytes(int n_rows, int n_phase);
}  // namespace soapgb
