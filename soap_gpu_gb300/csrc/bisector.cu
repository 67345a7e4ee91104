// Bisector injection of the seed spectra (the seed-cube preparation of
// CB_injection_faculae.py:191-244, BIS_inject_spectral_quiet / _active, with
// Delta_wavelength :119-123).  The reference runs it in Python: one pixel loop per
// spectrum and mu bin, then scipy's interp1d.  Here one launch computes the shifted
// grids of every mu bin, one checks that they increase, and one re-samples every
// (mu bin, pixel) with a binary search on its bin's grid.
//
// The arithmetic is the reference's, one rounding per operation (no contraction):
//   rv       = poly(f) (Horner from the highest power, as numpy.polyval) [+ vshift] * scale
//   wave_new = wave + wave (sqrt((1 + rv / c) / (1 - rv / c)) - 1)
//   out(x)   = f[j] if wave_new[j] == x, else ((f[j+1] - f[j]) / (wn[j+1] - wn[j])) (x - wn[j]) + f[j]
//              with wn[j] <= x < wn[j+1] -- numpy.interp, to which interp1d(kind='linear')
//              delegates for 1-D float64 data -- on the pixels strictly inside
//              (wave_new[0], wave_new[n-1]), 0 elsewhere.
// The reference's interp1d sorts a shifted grid that does not increase; here that is
// an error (status 61): it means the injected velocities fold the spectrum over.
#include "internal.cuh"

using namespace soapgb;

namespace {

constexpr int BIS_ST_ORDER = 61;
constexpr int BIS_MAX_COEF = 16;

__device__ __forceinline__ double bis_poly(const double *__restrict__ c, int n_coef, double x) {
    double y = 0.0;
    for (int q = 0; q < n_coef; ++q) y = __dadd_rn(__dmul_rn(y, x), c[q]);
    return y;
}

// shifted grids wn[b][k]; grid (ceil(n / 256), n_mu)
__global__ void k_bis_shift(int n, int n_coef, int mode, const double *__restrict__ wave,
                            const double *__restrict__ flux, const double *__restrict__ coeffs,
                            const double *__restrict__ coeffs_low, const double *__restrict__ dep_cut,
                            const double *__restrict__ vcut, const double *__restrict__ vshift, double scale,
                            double *__restrict__ wn) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (k >= n) return;
    const double f = flux[k], w = wave[k];
    double rv = 0.0;
    bool moved = true;
    if (mode == SOAPGB_BIS_QUIET) {
        rv = __dmul_rn(bis_poly(coeffs + (size_t)b * n_coef, n_coef, f), scale);
    } else {
        const double dc = dep_cut[b];
        if (f < dc && f > 0.5)
            rv = __dmul_rn(__dadd_rn(bis_poly(coeffs + (size_t)b * n_coef, n_coef, f), vshift[b]), scale);
        else if (f <= 0.5)
            rv = __dmul_rn(__dadd_rn(bis_poly(coeffs_low + (size_t)b * n_coef, n_coef, f), vshift[b]), scale);
        else if (f > dc)
            rv = __dmul_rn(__dadd_rn(vcut[b], vshift[b]), scale);
        else
            moved = false;
    }
    double out = w;
    if (moved) {
        const double beta = __ddiv_rn(rv, SOAP_C_LIGHT);
        const double r = __dsqrt_rn(__ddiv_rn(__dadd_rn(1.0, beta), __dsub_rn(1.0, beta)));
        out = __dadd_rn(w, __dmul_rn(w, __dsub_rn(r, 1.0)));
    }
    wn[(size_t)b * n + k] = out;
}

// every grid must increase strictly
__global__ void k_bis_order(int n, const double *__restrict__ wn, int *status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (k + 1 >= n) return;
    const double *g = wn + (size_t)b * n;
    if (!(g[k + 1] > g[k])) atomicExch(status, BIS_ST_ORDER);
}

// re-sampling at wave; grid (ceil(n / 256), n_mu)
__global__ void k_bis_resample(int n, const double *__restrict__ wave, const double *__restrict__ flux,
                               const double *__restrict__ wn, double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (i >= n) return;
    const double *g = wn + (size_t)b * n;
    const double x = wave[i];
    double y = 0.0;
    if (x > g[0] && x < g[n - 1]) {
        // the interval g[lo] <= x < g[lo + 1] (unique: g increases strictly, checked by
        // k_bis_order).  The shifted grid lies a few pixels from the unshifted one, so
        // a galloping search from i brackets it in O(log shift) loads, then bisection
        // inside the bracket [lo, hi] with g[lo] <= x < g[hi].
        int lo, hi;
        if (g[i] <= x) {
            lo = i;
            int step = 1;
            hi = min(n - 1, i + step);
            while (g[hi] <= x) {   // g[n - 1] > x ends it
                lo = hi;
                step <<= 1;
                hi = min(n - 1, lo + step);
            }
        } else {
            hi = i;
            int step = 1;
            lo = max(0, i - step);
            while (g[lo] > x) {    // g[0] < x ends it
                hi = lo;
                step <<= 1;
                lo = max(0, hi - step);
            }
        }
        while (hi - lo > 1) {
            const int mid = lo + ((hi - lo) >> 1);
            if (g[mid] <= x) lo = mid;
            else hi = mid;
        }
        if (g[lo] == x) {
            y = flux[lo];
        } else {
            const double slope = __ddiv_rn(__dsub_rn(flux[lo + 1], flux[lo]), __dsub_rn(g[lo + 1], g[lo]));
            y = __dadd_rn(__dmul_rn(slope, __dsub_rn(x, g[lo])), flux[lo]);
        }
    }
    out[(size_t)b * n + i] = y;
}

}  // namespace

extern "C" int soapgb_bisector_inject(soapgb_ctx *ctx, int mode, int n, int n_mu, int n_coef, const double *wave,
                                      const double *flux, const double *coeffs, const double *coeffs_low,
                                      const double *dep_cut, const double *vcut, const double *vshift,
                                      double scale, int mem, double *out) {
    if (!ctx) return SOAPGB_ERR_ARG;
    if (mode != SOAPGB_BIS_QUIET && mode != SOAPGB_BIS_ACTIVE)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_bisector_inject: unknown mode %d", mode);
    if (n < 2 || n_mu < 1 || n_coef < 1 || n_coef > BIS_MAX_COEF || !wave || !flux || !coeffs || !out)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_bisector_inject: bad arguments");
    if (mode == SOAPGB_BIS_ACTIVE && (!coeffs_low || !dep_cut || !vcut || !vshift))
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_bisector_inject: the active form needs coeffs_low, "
                                              "dep_cut, vcut and vshift");
    SOAP_DEVICE(ctx);
    const bool host = (mem == SOAPGB_HOST);
    const bool act = (mode == SOAPGB_BIS_ACTIVE);
    const size_t cube = sizeof(double) * (size_t)n * n_mu, row = sizeof(double) * (size_t)n;
    const size_t cb = sizeof(double) * (size_t)n_mu * n_coef, vb = sizeof(double) * (size_t)n_mu;
    Workspace ws(ctx);
    int s_wave = ws.add(host ? row : 0), s_flux = ws.add(host ? row : 0);
    int s_c = ws.add(host ? cb : 0), s_cl = ws.add(host && act ? cb : 0);
    int s_dc = ws.add(host && act ? vb : 0), s_vc = ws.add(host && act ? vb : 0), s_vs = ws.add(host && act ? vb : 0);
    int s_out = ws.add(host ? cube : 0);
    int s_wn = ws.add(cube);
    int rc = ws.commit();
    if (rc) return rc;
#define STAGE(dst, src, bytes, slot)                                               \
    dst = (decltype(dst))stage_in(ctx, mem, src, bytes, ws.get<void>(slot), &rc); \
    if (rc) return rc;
    const double *d_wave, *d_flux, *d_c, *d_cl = nullptr, *d_dc = nullptr, *d_vc = nullptr, *d_vs = nullptr;
    STAGE(d_wave, wave, row, s_wave);
    STAGE(d_flux, flux, row, s_flux);
    STAGE(d_c, coeffs, cb, s_c);
    if (act) {
        STAGE(d_cl, coeffs_low, cb, s_cl);
        STAGE(d_dc, dep_cut, vb, s_dc);
        STAGE(d_vc, vcut, vb, s_vc);
        STAGE(d_vs, vshift, vb, s_vs);
    }
#undef STAGE
    double *d_wn = ws.get<double>(s_wn);
    double *d_out = host ? ws.get<double>(s_out) : out;
    const dim3 g((n + 255) / 256, n_mu);
    SOAP_TRACED(ctx, "bis_shift", k_bis_shift<<<g, 256, 0, ctx->stream>>>(n, n_coef, mode, d_wave, d_flux, d_c, d_cl,
                                                                          d_dc, d_vc, d_vs, scale, d_wn));
    SOAP_LAUNCHED(ctx);
    k_bis_order<<<g, 256, 0, ctx->stream>>>(n, d_wn, ctx->d_status);
    SOAP_LAUNCHED(ctx);
    SOAP_TRACED(ctx, "bis_resample", k_bis_resample<<<g, 256, 0, ctx->stream>>>(n, d_wave, d_flux, d_wn, d_out));
    SOAP_LAUNCHED(ctx);
    if (!host) return SOAPGB_OK;
    SOAP_CUDA(ctx, cudaMemcpyAsync(out, d_out, cube, cudaMemcpyDeviceToHost, ctx->stream));
    SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return check_status(ctx, "soapgb_bisector_inject");
}
