// a11-a12: per-phase active-region integration.
//
// Reference: SOAP_integration.cu:392-447 (spot_integrate: a host loop over all
// G*G cells issuing eight FP64 kernels per active cell -- shift, three
// interpolations, intensity, flux/bconv/tot) and :285-323 (the accumulation
// kernels).  Here one launch covers every phase: block (x, p) owns a pixel range
// of phase p and gathers all of the phase's active cells, in map order, into
// register accumulators.
#include <cmath>

#include "internal.cuh"
#include "fir.cuh"

using namespace soapgb;

// loi_Planck, SOAP_integration.cu:205-212
__device__ __forceinline__ double soap_planck(double lambda0, double temp) {
    double c = 299792458.;
    double h = 6.62606896e-34;
    double k_b = 1.380e-23;
    double scale = 1e-10;
    return 2 * h * pow(c, 2) * 1. / pow(lambda0 * scale, 5) * 1. / (exp((h * c) / (lambda0 * k_b * temp * scale)) - 1);
}

constexpr int PHASE_CHUNK = 256;

// One cell's interpolation geometry at pixel j (shared by the three cubes).
struct CellAt {
    long long i;   // owner source index, -1 if none
    double dd;     // l'_{i+1} - l'_i
    double dl;     // l_j - l'_i
};

__device__ __forceinline__ CellAt soap_cell_at(long long j, int n_eff, const double *__restrict__ lam,
                                               const CellShift &c) {
    CellAt r;
    r.i = soap_owner(j, n_eff, c);
    r.dd = 0.0;
    r.dl = 0.0;
    if (r.i >= 0) {
        double li = lam[r.i], li1 = lam[r.i + 1];
        double ls0 = __dadd_rn(li, __dmul_rn(__dmul_rn(-1.0, li), __dsub_rn(1.0, c.sq)));
        double ls1 = __dadd_rn(li1, __dmul_rn(__dmul_rn(-1.0, li1), __dsub_rn(1.0, c.sq)));
        r.dd = __dsub_rn(ls1, ls0);
        r.dl = __dsub_rn(lam[j], ls0);
    }
    return r;
}

__device__ __forceinline__ double soap_lerp_at(const CellAt &a, long long j, const double *__restrict__ row,
                                               double delta, double limb) {
    if (delta == 0.0) return __dmul_rn(row[j], limb);
    if (a.i < 0) return 0.0;
    double s0 = row[a.i], s1 = row[a.i + 1];
    double t = __dmul_rn(__ddiv_rn(__dsub_rn(s1, s0), a.dd), a.dl);
    return __dmul_rn(__dadd_rn(s0, t), limb);
}

__global__ void __launch_bounds__(256) k_phase_plain64(
    int n, int n_eff, const double *__restrict__ lam, const double *__restrict__ q_norm,
    const double *__restrict__ q_sed, const double *__restrict__ spot_norm, const double *__restrict__ fac_norm,
    const double *__restrict__ spot_sed, const double *__restrict__ fac_sed, int max_cells,
    const int *__restrict__ cells, const int *__restrict__ counts, const double *__restrict__ temp,
    const double *__restrict__ bi, const double *__restrict__ delta_m, const double *__restrict__ limb_m,
    const double *__restrict__ lb_m, const int *__restrict__ region_m, long long gm, double step, int solar,
    int t_star, int t_diff_fac, double *__restrict__ flux, double *__restrict__ bconv, double *__restrict__ tot,
    long long out_stride, int n_mu, int *status) {
    __shared__ double s_delta[PHASE_CHUNK], s_limb[PHASE_CHUNK], s_fb[PHASE_CHUNK], s_sq[PHASE_CHUNK],
        s_off[PHASE_CHUNK], s_lb[PHASE_CHUNK], s_temp[PHASE_CHUNK];
    __shared__ int s_row[PHASE_CHUNK], s_type[PHASE_CHUNK];
    int p = blockIdx.y;
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double lambda0 = lam[0];
    const int *pc = cells + (long long)p * max_cells;
    int nc_all = counts[p];
    const double *pt = temp + (long long)p * gm;
    const double *pb = bi + (long long)p * gm;
    double fx = 0.0, bc = 0.0, tt = 0.0;
    double lj = (j < n_eff) ? lam[j] : 0.0;
    double ssed = (j < n_eff) ? spot_sed[j] : 0.0;
    double fsed = (j < n_eff) ? fac_sed[j] : 0.0;
    int t_norm_fac = (int)(t_star + t_diff_fac + 0.9 - 216.8);
    for (int c0 = 0; c0 < nc_all; c0 += PHASE_CHUNK) {
        int nc = min(PHASE_CHUNK, nc_all - c0);
        __syncthreads();
        for (int t = threadIdx.x; t < nc; t += blockDim.x) {
            int k = pc[c0 + t];
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
            s_lb[t] = lb_m[k];
            s_temp[t] = pt[k];
            s_type[t] = (pb[k] == 0.0) ? 0 : 1;
        }
        __syncthreads();
        if (j < n_eff) {
            for (int t = 0; t < nc; ++t) {
                CellShift cs;
                cs.fbeta = s_fb[t];
                cs.sq = s_sq[t];
                cs.off = s_off[t];
                double d = s_delta[t], L = s_limb[t];
                long long off = (long long)s_row[t] * n;
                CellAt at;
                if (d != 0.0) at = soap_cell_at(j, n_eff, lam, cs);
                double q = soap_lerp_at(at, j, q_norm + off, d, L);
                double s = soap_lerp_at(at, j, q_sed + off, d, L);
                double a, inten;
                if (s_type[t] == 0) {
                    // fast_intensity with T_norm = (int)T: the Planck ratio is exactly 1
                    double T = s_temp[t];
                    int tn = (int)T;
                    double ratio = ((double)tn == T) ? 1.0 : soap_planck(lj, T) / soap_planck(lj, (double)tn);
                    inten = __dmul_rn(ratio, ssed);
                    a = soap_lerp_at(at, j, spot_norm + off, d, L);
                } else {
                    if (solar) {
                        double T = s_temp[t];
                        double ratio = ((double)t_norm_fac == T) ? 1.0
                                                                  : soap_planck(lj, T) / soap_planck(lj, (double)t_norm_fac);
                        inten = __dmul_rn(ratio, fsed);
                    } else {
                        inten = __dmul_rn(__dadd_rn(1.0, s_lb[t]), fsed);
                    }
                    a = soap_lerp_at(at, j, fac_norm + off, d, L);
                }
                fx = __dsub_rn(__dadd_rn(fx, s), __dmul_rn(inten, q));
                bc = __dsub_rn(__dadd_rn(bc, q), a);
                tt = __dsub_rn(__dadd_rn(tt, s), __dmul_rn(a, inten));
            }
        }
    }
    long long o = (long long)p * out_stride + j;
    if (j < n_eff) {
        flux[o] = fx;
        bconv[o] = bc;
        tot[o] = tt;
    } else if (j < n) {
        flux[o] = 0.0;
        bconv[o] = 0.0;
        tot[o] = 0.0;
    }
}

// float -> double copy without FP64 instructions
__global__ void k_f32_widen(long long count, const float *__restrict__ a, double *__restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) out[i] = soap_f32_to_f64(a[i]);
}

namespace soapgb {

// Integration on device buffers (all pointers device).  temp/bi: n_phase x gm.
// out_stride: distance between phases in flux/bconv/tot (>= n).
// Outputs are float for the FP32 form (out_f32 must be set), double otherwise.
int integrate_device(soapgb_ctx *ctx, int form, int n, int n_eff, const double *d_wave, int grid, int n_phase,
                     const double *d_temp, const double *d_bi, const soapgb_maps &dm, const soapgb_cubes &dc,
                     double step, const soapgb_activity *act, void *d_flux, void *d_bconv, void *d_tot, int out_f32,
                     long long out_stride, int *d_cells, int *d_counts, char *fir_scratch,
                     const FirPlanSizes &fp) {
    if ((form == SOAPGB_FAST32) != (out_f32 != 0))
        return set_error(ctx, SOAPGB_ERR_ARG, "integration: FP32 outputs go with the FP32 form only");
    long long gm = (long long)grid * grid;
    if (form == SOAPGB_PLAIN64) {
        int rc = compact_cells(ctx, n_phase, (int)gm, d_bi, -0.5, 1.5, (int)gm, d_cells, d_counts);
        if (rc) return rc;
        dim3 g(grid_for(ctx, n, 256), n_phase);
        SOAP_TRACED(ctx, "integrate_plain64", k_phase_plain64<<<g, 256, 0, ctx->stream>>>(
            n, n_eff, d_wave, dc.q_norm, dc.q_sed, dc.spot_norm, dc.fac_norm, dc.spot_sed, dc.fac_sed, (int)gm,
            d_cells, d_counts, d_temp, d_bi, dm.delta, dm.limb, dm.lb, dm.region, gm, step, act->solar,
            act->t_star, act->t_diff_fac, (double *)d_flux, (double *)d_bconv, (double *)d_tot, out_stride, dc.n_mu,
            ctx->d_status));
        SOAP_LAUNCHED(ctx);
        return SOAPGB_OK;
    }
    FirPhaseArgs a;
    a.n = n;
    a.n_eff = n_eff;
    a.wave = d_wave;
    a.cubes = &dc;
    a.n_phase = n_phase;
    a.temp = d_temp;
    a.bi = d_bi;
    a.delta = dm.delta;
    a.limb = dm.limb;
    a.lb = dm.lb;
    a.region = dm.region;
    a.gm = gm;
    a.step = step;
    a.act = act;
    a.flux = d_flux;
    a.bconv = d_bconv;
    a.tot = d_tot;
    a.out_f32 = out_f32;
    a.out_stride = out_stride;
    return fir_phase(ctx, form, a, fir_scratch, fp);
}

}  // namespace soapgb

extern "C" int soapgb_phase_integrate(soapgb_ctx *ctx, int form, int n, int n_eff, const double *wave, int grid,
                                      int n_phase, const double *temp, const double *bi, const soapgb_maps *maps,
                                      const soapgb_cubes *cubes, double step, const soapgb_activity *act, int mem,
                                      double *flux, double *bconv, double *tot) {
    if (!ctx || !maps || !cubes || !act) return SOAPGB_ERR_ARG;
    if (n < 2 || n_eff < 2 || n_eff > n || grid < 1 || n_phase < 0 || cubes->n_mu < 1 || !(step > 0) || !wave ||
        !temp || !bi || !flux || !bconv || !tot || !maps->delta || !maps->limb || !maps->lb || !maps->region ||
        !cubes->q_norm || !cubes->q_sed || !cubes->spot_norm || !cubes->fac_norm || !cubes->spot_sed ||
        !cubes->fac_sed)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_phase_integrate: bad arguments");
    if (form != SOAPGB_PLAIN64 && form != SOAPGB_FAST64 && form != SOAPGB_FAST32)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_phase_integrate: unknown form %d", form);
    if (n_phase == 0) return SOAPGB_OK;
    SOAP_CUDA(ctx, cudaSetDevice(ctx->device));
    long long gm = (long long)grid * grid;
    int n_mu = cubes->n_mu;
    size_t cube_b = sizeof(double) * (size_t)n * n_mu;
    bool host = (mem == SOAPGB_HOST);
    Workspace ws(ctx);
    int s_wave = ws.add(host ? sizeof(double) * n : 0);
    int s_c[6];
    for (int q = 0; q < 4; ++q) s_c[q] = ws.add(host ? cube_b : 0);
    for (int q = 4; q < 6; ++q) s_c[q] = ws.add(host ? sizeof(double) * n : 0);
    int s_temp = ws.add(host ? sizeof(double) * gm * n_phase : 0);
    int s_bi = ws.add(host ? sizeof(double) * gm * n_phase : 0);
    int s_m[4];
    for (int q = 0; q < 3; ++q) s_m[q] = ws.add(host ? sizeof(double) * gm : 0);
    s_m[3] = ws.add(host ? sizeof(int) * gm : 0);
    int s_out[3];
    for (int q = 0; q < 3; ++q) s_out[q] = ws.add(host ? sizeof(double) * (size_t)n * n_phase : 0);
    int s_cells = ws.add(sizeof(int) * gm * n_phase);
    int s_counts = ws.add(sizeof(int) * n_phase);
    int s_f32 = ws.add(form == SOAPGB_FAST32 ? sizeof(float) * 3 * (size_t)n * n_phase : 0);
    FirPlanSizes fp = fir_plan_sizes(form, n, n_mu, gm, true, n_phase);
    int s_fir = ws.add(fp.bytes);
    int rc = ws.commit();
    if (rc) return rc;
#define STAGE(dst, src, bytes, slot)                                                           \
    dst = (decltype(dst))stage_in(ctx, mem, src, bytes, ws.get<void>(slot), &rc);             \
    if (rc) return rc;
    const double *d_wave;
    STAGE(d_wave, wave, sizeof(double) * n, s_wave);
    soapgb_cubes dc;
    dc.n_mu = n_mu;
    STAGE(dc.q_norm, cubes->q_norm, cube_b, s_c[0]);
    STAGE(dc.q_sed, cubes->q_sed, cube_b, s_c[1]);
    STAGE(dc.spot_norm, cubes->spot_norm, cube_b, s_c[2]);
    STAGE(dc.fac_norm, cubes->fac_norm, cube_b, s_c[3]);
    STAGE(dc.spot_sed, cubes->spot_sed, sizeof(double) * n, s_c[4]);
    STAGE(dc.fac_sed, cubes->fac_sed, sizeof(double) * n, s_c[5]);
    const double *d_temp, *d_bi;
    STAGE(d_temp, temp, sizeof(double) * gm * n_phase, s_temp);
    STAGE(d_bi, bi, sizeof(double) * gm * n_phase, s_bi);
    soapgb_maps dm;
    const double *cd;
    STAGE(cd, maps->delta, sizeof(double) * gm, s_m[0]);
    dm.delta = (double *)cd;
    STAGE(cd, maps->limb, sizeof(double) * gm, s_m[1]);
    dm.limb = (double *)cd;
    STAGE(cd, maps->lb, sizeof(double) * gm, s_m[2]);
    dm.lb = (double *)cd;
    const int *ci;
    STAGE(ci, maps->region, sizeof(int) * gm, s_m[3]);
    dm.region = (int *)ci;
    dm.mu = nullptr;
#undef STAGE
    double *d_flux = host ? ws.get<double>(s_out[0]) : flux;
    double *d_bconv = host ? ws.get<double>(s_out[1]) : bconv;
    double *d_tot = host ? ws.get<double>(s_out[2]) : tot;
    if (form == SOAPGB_FAST32) {
        float *f32 = ws.get<float>(s_f32);
        size_t pn = (size_t)n * n_phase;
        rc = integrate_device(ctx, form, n, n_eff, d_wave, grid, n_phase, d_temp, d_bi, dm, dc, step, act, f32,
                              f32 + pn, f32 + 2 * pn, 1, n, ws.get<int>(s_cells), ws.get<int>(s_counts),
                              ws.get<char>(s_fir), fp);
        if (rc) return rc;
        double *outs[3] = {d_flux, d_bconv, d_tot};
        for (int q = 0; q < 3; ++q) {
            SOAP_TRACED(ctx, "widen", k_f32_widen<<<grid_for(ctx, (long long)pn, 256), 256, 0, ctx->stream>>>((long long)pn, f32 + q * pn, outs[q]));
            SOAP_LAUNCHED(ctx);
        }
    } else {
        rc = integrate_device(ctx, form, n, n_eff, d_wave, grid, n_phase, d_temp, d_bi, dm, dc, step, act, d_flux,
                              d_bconv, d_tot, 0, n, ws.get<int>(s_cells), ws.get<int>(s_counts), ws.get<char>(s_fir),
                              fp);
        if (rc) return rc;
    }
    if (host) {
        size_t ob = sizeof(double) * (size_t)n * n_phase;
        SOAP_CUDA(ctx, cudaMemcpyAsync(flux, d_flux, ob, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(bconv, d_bconv, ob, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(tot, d_tot, ob, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return host ? check_status(ctx, "soapgb_phase_integrate") : SOAPGB_OK;
}
