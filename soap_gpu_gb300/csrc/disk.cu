// a3-a7: disk maps and the quiet-star disk integration.
//
// Reference: SOAP_initialize.cu:297-395 (itot) with fast_shift / fast_interp_new /
// fast_sum at :117-176.  The reference launches three kernels per visible cell
// (about 3 x 70,675 launches at G = 300) and scatters each cell into a scratch
// spectrum.  Here one launch sums all cells: every thread owns output pixels and
// gathers, for each cell in iy-major order, the source interval that covers the
// pixel (the interval-owning form of the scatter; see soap_owner()).
#include <cmath>
#include <vector>

#include "internal.cuh"
#include "fir.cuh"

using namespace soapgb;

// --------------------------------------------------------------------------
// a3: maps.  omega_velo (per iz) and sin(incl) come from the host, computed with
// the same libm calls as the reference's host loop; the rest is exact IEEE
// arithmetic, one rounding per operation.
// --------------------------------------------------------------------------
__global__ void k_disk_maps(int grid, const double *__restrict__ omega_velo, double sin_incl,
                            double delta_grid, double u1, double u2, int n_mu,
                            const double *__restrict__ mu_b, double lb0, double lb1, double lb2,
                            double lb3, double *delta_m, double *limb_m, double *mu_m,
                            int *region_m, double *lb_m) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long gm = (long long)grid * grid;
    if (k >= gm) return;
    int iy = (int)(k / grid), iz = (int)(k % grid);
    double y = __dadd_rn(-1., __dmul_rn((double)iy, delta_grid));
    double z = __dadd_rn(-1., __dmul_rn((double)iz, delta_grid));
    double delta = __dmul_rn(__dmul_rn(y, omega_velo[iz]), sin_incl);
    double d = -999.0, lm = -999.0, mu = -999.0, lb = -999.0;
    int reg = 0;
    double yz = __dadd_rn(__dmul_rn(y, y), __dmul_rn(z, z));
    if (yz <= 1.) {
        double r = __dsqrt_rn(__dsub_rn(1., yz));
        double om = __dsub_rn(1., r);
        lm = __dsub_rn(__dsub_rn(1., __dmul_rn(u1, om)), __dmul_rn(__dmul_rn(u2, om), om));
        lb = __dadd_rn(__dadd_rn(__dadd_rn(lb0, __dmul_rn(lb1, r)), __dmul_rn(__dmul_rn(lb2, r), r)),
                       __dmul_rn(__dmul_rn(__dmul_rn(lb3, r), r), r));
        reg = n_mu - 1;
        for (int b = 0; b < n_mu - 1; ++b)
            if (r > mu_b[b]) { reg = b; break; }
        d = delta;
        mu = r;
    }
    delta_m[k] = d;
    limb_m[k] = lm;
    mu_m[k] = mu;
    region_m[k] = reg;
    lb_m[k] = lb;
}

// --------------------------------------------------------------------------
// Ordered stream compaction: idx_out[list][...] = positions i (ascending) with
// lo <= key[list][i] <= hi.  One block of 1024 threads per list.
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_compact(const double *__restrict__ key, long long key_stride,
                                                  int n, double lo, double hi, int *idx_out,
                                                  int *count_out) {
    const double *kk = key + (long long)blockIdx.x * key_stride;
    int *out = idx_out + (long long)blockIdx.x * n;
    __shared__ int warp_tot[32];
    __shared__ int base;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    for (int start = 0; start < n; start += blockDim.x) {
        int i = start + threadIdx.x;
        bool p = false;
        if (i < n) {   // lo <= v <= hi by integer compares of the ordered bit patterns
            unsigned long long v = soap_ord64(kk[i]);
            p = (v >= soap_ord64(lo)) && (v <= soap_ord64(hi));
        }
        unsigned m = __ballot_sync(0xffffffffu, p);
        int pre = __popc(m & ((1u << lane) - 1u));
        if (lane == 0) warp_tot[w] = __popc(m);
        __syncthreads();
        if (w == 0) {
            int v = (lane < nw) ? warp_tot[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += t;
            }
            warp_tot[lane] = v;
        }
        __syncthreads();
        int woff = (w == 0) ? 0 : warp_tot[w - 1];
        if (p) out[base + woff + pre] = i;
        __syncthreads();
        if (threadIdx.x == 0) base += warp_tot[nw - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) count_out[blockIdx.x] = base;
}

namespace soapgb {
int compact_cells(soapgb_ctx *ctx, int n_lists, int cells_per_list, const double *key, double lo,
                  double hi, int key_stride, int *idx_out, int *count_out) {
    SOAP_TRACED(ctx, "compact", k_compact<<<n_lists, 1024, 0, ctx->stream>>>(key, key_stride, cells_per_list, lo, hi, idx_out,
                                                  count_out));
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}
}  // namespace soapgb

// --------------------------------------------------------------------------
// a4-a7 plain FP64: per-pixel gather over all visible cells, in map order.
// The arithmetic of one (cell, pixel) term is the reference's:
//   (S[i] + (S[i+1]-S[i]) / (l'_{i+1} - l'_i) * (l_j - l'_i)) * limb
// with one IEEE rounding per operation (no contraction), so the sum is bit-equal
// to a sequential CPU loop over cells.
// --------------------------------------------------------------------------
constexpr int QUIET_CHUNK = 512;

__device__ __forceinline__ double soap_cell_value(long long j, int n_eff, const double *__restrict__ lam,
                                                  const double *__restrict__ row, double delta,
                                                  double limb, const CellShift &c) {
    if (delta == 0.0) return __dmul_rn(row[j], limb);
    long long i = soap_owner(j, n_eff, c);
    if (i < 0) return 0.0;
    double li = lam[i], li1 = lam[i + 1];
    double ls0 = __dadd_rn(li, __dmul_rn(__dmul_rn(-1.0, li), __dsub_rn(1.0, c.sq)));
    double ls1 = __dadd_rn(li1, __dmul_rn(__dmul_rn(-1.0, li1), __dsub_rn(1.0, c.sq)));
    double s0 = row[i], s1 = row[i + 1];
    double g = __dsub_rn(s1, s0);
    double dd = __dsub_rn(ls1, ls0);
    double t = __dmul_rn(__ddiv_rn(g, dd), __dsub_rn(lam[j], ls0));
    return __dmul_rn(__dadd_rn(s0, t), limb);
}

__global__ void __launch_bounds__(256) k_quiet_plain64(int n, int n_eff, const double *__restrict__ lam,
                                                       const double *__restrict__ cube,
                                                       const int *__restrict__ n_cells_ptr,
                                                       const int *__restrict__ cells,
                                                       const double *__restrict__ delta_m,
                                                       const double *__restrict__ limb_m,
                                                       const int *__restrict__ region_m, double step, int n_mu,
                                                       double *__restrict__ out, int *status) {
    __shared__ double s_delta[QUIET_CHUNK], s_limb[QUIET_CHUNK], s_fb[QUIET_CHUNK], s_sq[QUIET_CHUNK],
        s_off[QUIET_CHUNK];
    __shared__ int s_row[QUIET_CHUNK];
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double lambda0 = lam[0];
    double sum = 0.0;
    int n_cells = *n_cells_ptr;
    for (int c0 = 0; c0 < n_cells; c0 += QUIET_CHUNK) {
        int nc = min(QUIET_CHUNK, n_cells - c0);
        __syncthreads();
        for (int t = threadIdx.x; t < nc; t += blockDim.x) {
            int k = cells[c0 + t];
            double d = delta_m[k];
            CellShift cs = soap_cell_shift(d, lambda0, step);
            s_delta[t] = d;
            s_limb[t] = limb_m[k];
            s_fb[t] = cs.fbeta;
            s_sq[t] = cs.sq;
            s_off[t] = cs.off;
            int row = region_m[k];
            if ((unsigned)row >= (unsigned)n_mu) {   // mu bin outside the cube: report, use bin 0
                atomicExch(status, 21);
                row = 0;
            }
            s_row[t] = row;
        }
        __syncthreads();
        if (j < n_eff) {
            for (int t = 0; t < nc; ++t) {
                CellShift cs;
                cs.fbeta = s_fb[t];
                cs.sq = s_sq[t];
                cs.off = s_off[t];
                const double *row = cube + (long long)s_row[t] * n;
                sum = __dadd_rn(sum, soap_cell_value(j, n_eff, lam, row, s_delta[t], s_limb[t], cs));
            }
        }
    }
    if (j < n_eff) out[j] = sum;
    else if (j < n) out[j] = 0.0;
}

// --------------------------------------------------------------------------
// host side
// --------------------------------------------------------------------------
namespace soapgb {
void disk_omega_host(const soapgb_star *st, std::vector<double> &ov, double &sin_incl);
int disk_maps_launch(soapgb_ctx *ctx, const soapgb_star *star, int n_mu, const double *d_mu, const double *d_ov,
                     double sin_incl, double *delta, double *limb, double *mu, int *region, double *lb);
}  // namespace soapgb

static void host_omega_velo(const soapgb_star *st, std::vector<double> &ov, double &sin_incl) {
    // SOAP_initialize.cu:308-351, host libm like the reference
    double incl = st->incl * SOAP_PI / 180.;
    double theta_grid = 180.0 / st->grid;
    double omega0 = 360.0 / st->period;
    double omega1 = omega0 * st->omega_ratio;
    ov.resize(st->grid);
    for (int iz = 0; iz < st->grid; ++iz) {
        double theta_z = -90.0 + iz * theta_grid;
        double s = sin(theta_z * SOAP_PI / 180);
        ov[iz] = (omega0 + omega1 * (s * s)) * SOAP_PI / (180 * 24 * 3600) * st->radius_km;
    }
    sin_incl = sin(incl);
}

namespace soapgb {
// the per-row rotation constants of a star's grid (host libm), for disk_maps_launch
void disk_omega_host(const soapgb_star *st, std::vector<double> &ov, double &sin_incl) {
    host_omega_velo(st, ov, sin_incl);
}

// the disk maps of one star from constants already on the device (no host memory read)
int disk_maps_launch(soapgb_ctx *ctx, const soapgb_star *star, int n_mu, const double *d_mu, const double *d_ov,
                     double sin_incl, double *delta, double *limb, double *mu, int *region, double *lb) {
    const int G = star->grid;
    const long long gm = (long long)G * G;
    const double *c = star->lb;
    SOAP_TRACED(ctx, "disk_maps", k_disk_maps<<<grid_for(ctx, gm, 256), 256, 0, ctx->stream>>>(
        G, d_ov, sin_incl, 2. / G, star->u1, star->u2, n_mu, d_mu, c[0], c[1], c[2], c[3], delta, limb, mu, region,
        lb));
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}
}  // namespace soapgb

extern "C" int soapgb_disk_maps(soapgb_ctx *ctx, const soapgb_star *star, int n_mu,
                                const double *mu_boundary, int mem, soapgb_maps *maps_out) {
    if (!ctx || !star || !maps_out) return SOAPGB_ERR_ARG;
    if (star->grid <= 0 || star->grid > 20000 || n_mu < 1 || (n_mu > 1 && !mu_boundary))
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_disk_maps: bad grid %d / n_mu %d", star->grid, n_mu);
    SOAP_DEVICE(ctx);
    int G = star->grid;
    long long gm = (long long)G * G;
    std::vector<double> ov;
    double sin_incl;
    host_omega_velo(star, ov, sin_incl);
    Workspace ws(ctx);
    int s_ov = ws.add(sizeof(double) * G);
    int s_mu = ws.add(sizeof(double) * (n_mu > 1 ? n_mu - 1 : 1));
    int s_out[5];
    for (int q = 0; q < 5; ++q) s_out[q] = ws.add(mem == SOAPGB_HOST ? sizeof(double) * gm : 0);
    int rc = ws.commit();
    if (rc) return rc;
    double *d_ov = ws.get<double>(s_ov);
    SOAP_CUDA(ctx, cudaMemcpyAsync(d_ov, ov.data(), sizeof(double) * G, cudaMemcpyHostToDevice, ctx->stream));
    const double *d_mu = mu_boundary;
    if (n_mu > 1 && mem == SOAPGB_HOST) {
        d_mu = ws.get<double>(s_mu);
        SOAP_CUDA(ctx, cudaMemcpyAsync((void *)d_mu, mu_boundary, sizeof(double) * (n_mu - 1),
                                       cudaMemcpyHostToDevice, ctx->stream));
    }
    double *o_delta = maps_out->delta, *o_limb = maps_out->limb, *o_mu = maps_out->mu, *o_lb = maps_out->lb;
    int *o_reg = maps_out->region;
    if (mem == SOAPGB_HOST) {
        o_delta = ws.get<double>(s_out[0]);
        o_limb = ws.get<double>(s_out[1]);
        o_mu = ws.get<double>(s_out[2]);
        o_lb = ws.get<double>(s_out[3]);
        o_reg = ws.get<int>(s_out[4]);
    }
    if (!o_delta || !o_limb || !o_mu || !o_lb || !o_reg)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_disk_maps: null map pointer");
    const double *lb = star->lb;
    SOAP_TRACED(ctx, "disk_maps", k_disk_maps<<<grid_for(ctx, gm, 256), 256, 0, ctx->stream>>>(
        G, d_ov, sin_incl, 2. / G, star->u1, star->u2, n_mu, d_mu, lb[0], lb[1], lb[2], lb[3], o_delta, o_limb,
        o_mu, o_reg, o_lb));
    SOAP_LAUNCHED(ctx);
    if (mem == SOAPGB_HOST) {
        SOAP_CUDA(ctx, cudaMemcpyAsync(maps_out->delta, o_delta, sizeof(double) * gm, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(maps_out->limb, o_limb, sizeof(double) * gm, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(maps_out->mu, o_mu, sizeof(double) * gm, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(maps_out->lb, o_lb, sizeof(double) * gm, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(maps_out->region, o_reg, sizeof(int) * gm, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return SOAPGB_OK;
}

extern "C" int soapgb_quiet_disk(soapgb_ctx *ctx, int form, int n, int n_eff, const double *wave,
                                 const double *cube, int n_mu, int grid, const double *delta,
                                 const double *limb, const int *region, double step, int mem,
                                 double *sum_out) {
    if (!ctx) return SOAPGB_ERR_ARG;
    if (n < 2 || n_eff < 2 || n_eff > n || n_mu < 1 || grid < 1 || !wave || !cube || !delta || !limb ||
        !region || !sum_out || !(step > 0))
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_quiet_disk: bad arguments (n=%d n_eff=%d)", n, n_eff);
    if (form != SOAPGB_PLAIN64 && form != SOAPGB_FAST64 && form != SOAPGB_FAST32)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_quiet_disk: unknown form %d", form);
    SOAP_DEVICE(ctx);
    long long gm = (long long)grid * grid;
    bool host = (mem == SOAPGB_HOST);
    Workspace ws(ctx);
    int s_wave = ws.add(host ? sizeof(double) * n : 0);
    int s_cube = ws.add(host ? sizeof(double) * (size_t)n * n_mu : 0);
    int s_delta = ws.add(host ? sizeof(double) * gm : 0);
    int s_limb = ws.add(host ? sizeof(double) * gm : 0);
    int s_region = ws.add(host ? sizeof(int) * gm : 0);
    int s_out = ws.add(host ? sizeof(double) * n : 0);
    int s_cells = ws.add(sizeof(int) * gm);
    int s_count = ws.add(sizeof(int));
    FirPlanSizes fp = fir_plan_sizes(form, n, n_mu, gm, false, 1);
    int s_fir = ws.add(fp.bytes);
    int rc = ws.commit();
    if (rc) return rc;
    const double *d_wave = (const double *)stage_in(ctx, mem, wave, sizeof(double) * n, ws.get<void>(s_wave), &rc);
    if (rc) return rc;
    const double *d_cube = (const double *)stage_in(ctx, mem, cube, sizeof(double) * (size_t)n * n_mu, ws.get<void>(s_cube), &rc);
    if (rc) return rc;
    const double *d_delta = (const double *)stage_in(ctx, mem, delta, sizeof(double) * gm, ws.get<void>(s_delta), &rc);
    if (rc) return rc;
    const double *d_limb = (const double *)stage_in(ctx, mem, limb, sizeof(double) * gm, ws.get<void>(s_limb), &rc);
    if (rc) return rc;
    const int *d_region = (const int *)stage_in(ctx, mem, region, sizeof(int) * gm, ws.get<void>(s_region), &rc);
    if (rc) return rc;
    double *d_out = host ? ws.get<double>(s_out) : sum_out;
    int *d_cells = ws.get<int>(s_cells);
    int *d_count = ws.get<int>(s_count);
    if (form == SOAPGB_PLAIN64) {
        // visible cells in map order (limb map is -999 elsewhere)
        rc = compact_cells(ctx, 1, (int)gm, d_limb, -998.0, 1e300, (int)gm, d_cells, d_count);
        if (rc) return rc;
        SOAP_TRACED(ctx, "quiet_plain64", k_quiet_plain64<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, n_eff, d_wave, d_cube, d_count, d_cells,
                                                                         d_delta, d_limb, d_region, step, n_mu, d_out,
                                                                         ctx->d_status));
        SOAP_LAUNCHED(ctx);
    } else {
        FirQuietArgs qa;
        qa.n = n;
        qa.n_eff = n_eff;
        qa.wave = d_wave;
        qa.cube = d_cube;
        qa.n_mu = n_mu;
        qa.gm = gm;
        qa.delta = d_delta;
        qa.limb = d_limb;
        qa.region = d_region;
        qa.step = step;
        qa.out = d_out;
        rc = fir_quiet(ctx, form, qa, ws.get<char>(s_fir), fp);
        if (rc) return rc;
    }
    if (host) {
        SOAP_CUDA(ctx, cudaMemcpyAsync(sum_out, d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return host ? check_status(ctx, "soapgb_quiet_disk") : SOAPGB_OK;
}
