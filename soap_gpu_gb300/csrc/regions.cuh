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

namespace soapgb {
// The region table of n_phase phases built on the host and copied to scratch:
// *d_table (reg_off[n_phase] rows) and *d_off (n_phase + 1 offsets); phase_visible
// (optional) gets 1 for the phases with at least one visible region, else 0.
int phase_table_device(soapgb_ctx *ctx, int grid, double incl, int n_phase, const double *h_phases,
                       const int *h_reg_off, const double *h_regions, const soapgb_activity *act, char *scratch,
                       size_t scratch_bytes, const RegionPhase **d_table, const int **d_off,
                       std::vector<unsigned char> *phase_visible = nullptr);
size_t phase_maps_scratch_bytes(int n_rows, int n_phase);
}  // namespace soapgb
