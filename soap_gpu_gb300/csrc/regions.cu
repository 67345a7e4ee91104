// a9-a10: per-phase active-region maps.
//
// Reference: SOAP_integration.cu:21-161 (spot_init_gpu, spot_phase_gpu, spot_area:
// three launches of nrho x 3 threads plus a device-to-host copy per region and
// phase) and :326-390 (spot_scan, a host loop over the bounding box).  Here the
// per-(phase, region) constants -- the rim's bounding box and the inverse rotation
// -- are a few hundred libm calls done on the host, and one launch scans every
// cell of every phase, applying the regions in order (later regions overwrite).
// The rim bounding box is computed from all nrho points at once, which is the
// deterministic form of spot_area's cross-block reduction (:61-93).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "regions.cuh"

using namespace soapgb;

// spot_init_gpu + spot_phase_gpu + spot_area for one region at one phase
static void host_region_bbox(double s, double longitude, double latitude, double inclination, int nrho,
                             double phase, int grid, int *bounds) {
    double lon = longitude * SOAP_PI / 180.;
    double lat = latitude * SOAP_PI / 180.;
    double inc = inclination * SOAP_PI / 180.;
    double rho_step = 2. * SOAP_PI / (nrho - 1);
    double b = -lat, g = lon, b2 = SOAP_PI / 2. - inc;
    double R[3][3] = {{cos(b2) * cos(g) * cos(b) - sin(b) * sin(b2), -sin(g) * cos(b2), cos(b2) * cos(g) * sin(b) + sin(b2) * cos(b)},
                      {sin(g) * cos(b), cos(g), sin(g) * sin(b)},
                      {-sin(b2) * cos(g) * cos(b) - cos(b2) * sin(b), sin(b2) * sin(g), -sin(b2) * cos(g) * sin(b) + cos(b2) * cos(b)}};
    double psi = -phase * (2 * SOAP_PI);
    double axe[3] = {cos(inc), 0, sin(inc)};
    double cp = cos(psi), sp = sin(psi);
    double P[3][3] = {{(1 - cp) * axe[0] * axe[0] + cp, (1 - cp) * axe[0] * axe[1] + sp * axe[2], (1 - cp) * axe[0] * axe[2] - sp * axe[1]},
                      {(1 - cp) * axe[1] * axe[0] - sp * axe[2], (1 - cp) * axe[1] * axe[1] + cp, (1 - cp) * axe[1] * axe[2] + sp * axe[0]},
                      {(1 - cp) * axe[2] * axe[0] + sp * axe[1], (1 - cp) * axe[2] * axe[1] - sp * axe[0], (1 - cp) * axe[2] * axe[2] + cp}};
    double grid_step = 2. / grid;
    double miny = 1, minz = 1, maxy = -1, maxz = -1;
    int sum_on = 0, sum_off = 0;
    for (int k = 0; k < nrho; k++) {
        double rho = -SOAP_PI + k * rho_step;
        double x2[3] = {sqrt(1 - s * s), s * cos(rho), s * sin(rho)};
        double x1[3], x3[3];
        for (int r = 0; r < 3; r++) x1[r] = R[r][0] * x2[0] + R[r][1] * x2[1] + R[r][2] * x2[2];
        for (int r = 0; r < 3; r++) x3[r] = P[r][0] * x1[0] + P[r][1] * x1[1] + P[r][2] * x1[2];
        if (x3[0] >= 0) {
            sum_on++;
            if (x3[1] < miny) miny = x3[1];
            if (x3[2] < minz) minz = x3[2];
            if (x3[1] > maxy) maxy = x3[1];
            if (x3[2] > maxz) maxz = x3[2];
        } else {
            sum_off++;
        }
    }
    if ((sum_on > 0) && (sum_off > 0)) {
        if (miny * maxy < 0) { if (minz < 0) minz = -1; else maxz = 1; }
        if (minz * maxz < 0) { if (miny < 0) miny = -1; else maxy = 1; }
    }
    bounds[0] = (int)floor((1. + miny) / grid_step);
    bounds[1] = (int)floor((1. + minz) / grid_step);
    bounds[2] = (int)ceil((1. + maxy) / grid_step);
    bounds[3] = (int)ceil((1. + maxz) / grid_step);
    bounds[4] = sum_on == 0 ? 0 : 1;
}

// spot_inverse_rotation, SOAP_integration.cu:164-202 (note `--phase`: the phase
// is decremented by one before the multiply); first row of R2 * R only.
static void host_inverse_row0(double longitude, double latitude, double inclination, double phase, double *row) {
    double g2 = (phase - 1.0) * (2 * SOAP_PI);
    double i = inclination * SOAP_PI / 180.;
    double b = latitude * SOAP_PI / 180.;
    double g = -longitude * SOAP_PI / 180.;
    double b2 = -(SOAP_PI / 2. - i);
    double R[3][3] = {{(1 - cos(g2)) * cos(i) * cos(i) + cos(g2), sin(g2) * sin(i), (1 - cos(g2)) * cos(i) * sin(i)},
                      {-sin(g2) * sin(i), cos(g2), sin(g2) * cos(i)},
                      {(1 - cos(g2)) * sin(i) * cos(i), -sin(g2) * cos(i), (1 - cos(g2)) * sin(i) * sin(i) + cos(g2)}};
    double R2[3][3] = {{cos(b) * cos(g) * cos(b2) - sin(b2) * sin(b), -sin(g) * cos(b), cos(b) * cos(g) * sin(b2) + sin(b) * cos(b2)},
                       {sin(g) * cos(b2), cos(g), sin(g) * sin(b2)},
                       {-sin(b) * cos(g) * cos(b2) - cos(b) * sin(b2), sin(b) * sin(g), -sin(b) * cos(g) * sin(b2) + cos(b) * cos(b2)}};
    for (int q = 0; q < 3; q++) row[q] = R2[0][0] * R[0][q] + R2[0][1] * R[1][q] + R2[0][2] * R[2][q];
}

__global__ void k_phase_scan(int grid, double delta_grid, const RegionPhase *__restrict__ table,
                             const int *__restrict__ reg_off, int t_star, int t_diff_spot, int t_diff_fac,
                             double *temp, double *bi) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long gm = (long long)grid * grid;
    int p = blockIdx.y;
    if (k >= gm) return;
    int iy = (int)(k / grid), iz = (int)(k % grid);
    double t, b;
    region_cell_value(table, reg_off[p], reg_off[p + 1], iy, iz, delta_grid, t_star, t_diff_spot, t_diff_fac, t, b);
    temp[(long long)p * gm + k] = t;
    bi[(long long)p * gm + k] = b;
}

// Builds the per-(phase, region) table on the host.  phases/regions/offsets are host arrays.
static int build_region_table(soapgb_ctx *ctx, int grid, double incl, int n_phase, const double *phases,
                              const int *reg_off, const double *regions, int nrho,
                              std::vector<RegionPhase> &table) {
    if (nrho < 2) return set_error(ctx, SOAPGB_ERR_ARG, "nrho must be >= 2 (got %d)", nrho);
    if (reg_off[0] != 0) return set_error(ctx, SOAPGB_ERR_ARG, "reg_offsets[0] must be 0");
    int n_rows = reg_off[n_phase];
    table.resize(n_rows > 0 ? n_rows : 1);
    for (int p = 0; p < n_phase; ++p) {
        if (reg_off[p + 1] < reg_off[p]) return set_error(ctx, SOAPGB_ERR_ARG, "reg_offsets not ascending");
        for (int r = reg_off[p]; r < reg_off[p + 1]; ++r) {
            const double *row = regions + 4 * (size_t)r;
            double lat = row[0], lon = row[1], s = row[2], type = row[3];
            if (!(s >= 0.0 && s < 1.0))
                return set_error(ctx, SOAPGB_ERR_ARG, "region size must be in [0, 1) (got %g)", s);
            int bd[5];
            host_region_bbox(s, lon, lat, incl, nrho, phases[p], grid, bd);
            RegionPhase &rp = table[r];
            rp.iy0 = bd[0] < 0 ? 0 : bd[0];
            rp.iz0 = bd[1] < 0 ? 0 : bd[1];
            rp.iy1 = bd[2] > grid ? grid : bd[2];
            rp.iz1 = bd[3] > grid ? grid : bd[3];
            rp.visible = bd[4];
            rp.type = (type == 0.0) ? 0 : 1;
            rp.s = s;
            double r3[3];
            host_inverse_row0(lon, lat, incl, phases[p], r3);
            rp.r0 = r3[0];
            rp.r1 = r3[1];
            rp.r2 = r3[2];
            // the FP32 owner test's constants (its margins absorb their rounding)
            rp.f0 = (float)rp.r0;
            rp.f1 = (float)rp.r1;
            rp.f2 = (float)rp.r2;
            rp.fcap = (float)(1.0 - s * s);
        }
    }
    return SOAPGB_OK;
}

namespace soapgb {
int phase_table_device(soapgb_ctx *ctx, int grid, double incl, int n_phase, const double *h_phases,
                       const int *h_reg_off, const double *h_regions, const soapgb_activity *act, char *scratch,
                       size_t scratch_bytes, const RegionPhase **d_table, const int **d_off,
                       std::vector<unsigned char> *phase_visible, long long *max_box_cells,
                       std::vector<char> *pack) {
    std::vector<RegionPhase> table;
    int rc = build_region_table(ctx, grid, incl, n_phase, h_phases, h_reg_off, h_regions, act->nrho, table);
    if (rc) return rc;
    if (phase_visible) {
        phase_visible->assign(n_phase, 0);
        for (int p = 0; p < n_phase; ++p)
            for (int r = h_reg_off[p]; r < h_reg_off[p + 1]; ++r)
                if (table[r].visible) (*phase_visible)[p] = 1;
    }
    if (max_box_cells) {
        long long mx = 0;
        for (int p = 0; p < n_phase; ++p) {
            long long sum = 0;
            for (int r = h_reg_off[p]; r < h_reg_off[p + 1]; ++r) {
                const RegionPhase &t = table[r];
                if (t.visible && t.iy1 > t.iy0 && t.iz1 > t.iz0) sum += (long long)(t.iy1 - t.iy0) * (t.iz1 - t.iz0);
            }
            mx = std::max(mx, sum);
        }
        *max_box_cells = mx;
    }
    size_t tb = sizeof(RegionPhase) * table.size();
    size_t ob = sizeof(int) * (n_phase + 1);
    if (((tb + 255) & ~size_t(255)) + ob > scratch_bytes)
        return set_error(ctx, SOAPGB_ERR_ARG, "phase maps scratch too small");
    RegionPhase *dt = (RegionPhase *)scratch;
    int *dof = (int *)(scratch + ((tb + 255) & ~size_t(255)));
    if (pack) {   // the caller copies the scratch image in one go
        pack->assign(((tb + 255) & ~size_t(255)) + ob, 0);
        memcpy(pack->data(), table.data(), tb);
        memcpy(pack->data() + ((tb + 255) & ~size_t(255)), h_reg_off, ob);
    } else {
        SOAP_CUDA(ctx, cudaMemcpyAsync(dt, table.data(), tb, cudaMemcpyHostToDevice, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(dof, h_reg_off, ob, cudaMemcpyHostToDevice, ctx->stream));
        // `table` lives in pageable memory: cudaMemcpyAsync has staged it before returning
    }
    *d_table = dt;
    *d_off = dof;
    return SOAPGB_OK;
}

// Device-side phase maps for already-device temp/bi outputs; phases/regions/offsets on host.
int phase_maps_device(soapgb_ctx *ctx, int grid, double incl, int n_phase, const double *h_phases,
                      const int *h_reg_off, const double *h_regions, const soapgb_activity *act, double *d_temp,
                      double *d_bi, char *scratch, size_t scratch_bytes) {
    const RegionPhase *d_table;
    const int *d_off;
    int rc = phase_table_device(ctx, grid, incl, n_phase, h_phases, h_reg_off, h_regions, act, scratch, scratch_bytes,
                                &d_table, &d_off);
    if (rc) return rc;
    long long gm = (long long)grid * grid;
    dim3 g(grid_for(ctx, gm, 256), n_phase);
    SOAP_TRACED(ctx, "phase_scan", k_phase_scan<<<g, 256, 0, ctx->stream>>>(grid, 2. / grid, d_table, d_off, act->t_star, act->t_diff_spot,
                                             act->t_diff_fac, d_temp, d_bi));
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}

size_t phase_maps_scratch_bytes(int n_rows, int n_phase) {
    size_t tb = sizeof(RegionPhase) * (size_t)(n_rows > 0 ? n_rows : 1);
    return ((tb + 255) & ~size_t(255)) + sizeof(int) * (n_phase + 1) + 256;
}
}  // namespace soapgb

extern "C" int soapgb_phase_maps(soapgb_ctx *ctx, int grid, double incl, int n_phase, const double *phases,
                                 const int *reg_offsets, const double *regions, const soapgb_activity *act,
                                 int mem, double *temp, double *bi) {
    if (!ctx || !act) return SOAPGB_ERR_ARG;
    if (grid < 1 || grid > 20000 || n_phase < 0 || !phases || !reg_offsets || !temp || !bi)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_phase_maps: bad arguments");
    if (n_phase == 0) return SOAPGB_OK;
    SOAP_DEVICE(ctx);
    // bring the (small) phase / region description to the host
    std::vector<int> h_off(n_phase + 1);
    std::vector<double> h_ph(n_phase);
    if (mem == SOAPGB_DEVICE) {
        SOAP_CUDA(ctx, cudaMemcpyAsync(h_off.data(), reg_offsets, sizeof(int) * (n_phase + 1), cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(h_ph.data(), phases, sizeof(double) * n_phase, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    } else {
        memcpy(h_off.data(), reg_offsets, sizeof(int) * (n_phase + 1));
        memcpy(h_ph.data(), phases, sizeof(double) * n_phase);
    }
    int n_rows = h_off[n_phase];
    if (n_rows < 0) return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_phase_maps: negative region count");
    std::vector<double> h_reg(4 * (size_t)(n_rows > 0 ? n_rows : 1));
    if (n_rows > 0) {
        if (!regions) return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_phase_maps: null regions");
        if (mem == SOAPGB_DEVICE) {
            SOAP_CUDA(ctx, cudaMemcpyAsync(h_reg.data(), regions, sizeof(double) * 4 * n_rows, cudaMemcpyDeviceToHost, ctx->stream));
            SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        } else {
            memcpy(h_reg.data(), regions, sizeof(double) * 4 * n_rows);
        }
    }
    long long gm = (long long)grid * grid;
    bool host = (mem == SOAPGB_HOST);
    Workspace ws(ctx);
    int s_scr = ws.add(phase_maps_scratch_bytes(n_rows, n_phase));
    int s_t = ws.add(host ? sizeof(double) * gm * n_phase : 0);
    int s_b = ws.add(host ? sizeof(double) * gm * n_phase : 0);
    int rc = ws.commit();
    if (rc) return rc;
    double *d_t = host ? ws.get<double>(s_t) : temp;
    double *d_b = host ? ws.get<double>(s_b) : bi;
    rc = phase_maps_device(ctx, grid, incl, n_phase, h_ph.data(), h_off.data(), h_reg.data(), act, d_t, d_b,
                           ws.get<char>(s_scr), phase_maps_scratch_bytes(n_rows, n_phase));
    if (rc) return rc;
    if (host) {
        SOAP_CUDA(ctx, cudaMemcpyAsync(temp, d_t, sizeof(double) * gm * n_phase, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(bi, d_b, sizeof(double) * gm * n_phase, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return SOAPGB_OK;
}
