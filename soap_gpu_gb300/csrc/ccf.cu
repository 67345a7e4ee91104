// a15-a16: binary-mask CCF.
//
// Reference: CCF_func.py:5-36 (calculate_CCF_1 builds a dense n_v x n_w mask with
// Python loops over velocities and lines; calculate_CCF_2 takes n_v dense dot
// products per spectrum) and :39-91 (calc_mask), on the extended grid of
// run_all_SOAP.py:292-295.  Here the mask is built once per call on the device
// and kept sparse (about four entries per line and velocity), with the
// reference's "later line overwrites" rule resolved by a max-sequence pass; the
// dot products for all spectra then read only the mask's entries.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.cuh"

using namespace soapgb;

struct CcfGeom {
    double start_b, stop_b;   // linspace before the grid
    double start_a, stop_a;   // linspace after the grid
    double begin_wave;        // wavelength_extend.min()
    double k_hw;              // sqrt((1+b)/(1-b)) - 1 for the 820 m/s hole
    int np_ext, n_ext, n_w, index_old;
    double mask_step;
};

// wavelength_extend[k] (numpy.linspace: k*step + start, last element = stop)
__device__ __forceinline__ double ccf_we(const CcfGeom &g, const double *__restrict__ wt, long long k) {
    if (k < g.np_ext) {
        if (k == g.np_ext - 1) return g.stop_b;
        double st = __ddiv_rn(__dsub_rn(g.stop_b, g.start_b), (double)(g.np_ext - 1));
        return __dadd_rn(__dmul_rn((double)k, st), g.start_b);
    }
    if (k < g.np_ext + g.n_w) return wt[k - g.np_ext];
    long long q = k - g.np_ext - g.n_w;
    if (q == g.np_ext - 1) return g.stop_a;
    double st = __ddiv_rn(__dsub_rn(g.stop_a, g.start_a), (double)(g.np_ext - 1));
    return __dadd_rn(__dmul_rn((double)q, st), g.start_a);
}

struct LineWin {
    long long aa, bb;     // hole pixel range: [aa, bb) full weight, aa-1 and bb fractional
    double w, frb, fra;
    int ok;
};

// calc_mask for one (velocity, line), CCF_func.py:48-89
__device__ __forceinline__ LineWin ccf_line(const CcfGeom &g, const double *__restrict__ wt, double v,
                                            double lw, double weight) {
    LineWin r;
    double fac = __dadd_rn(1.0, __ddiv_rn(v, SOAP_C_LIGHT));
    double ls = __dmul_rn(lw, fac);
    double hw = __dmul_rn(ls, g.k_hw);
    double beg = __dsub_rn(ls, __ddiv_rn(hw, 2.0));
    double end = __dadd_rn(ls, __ddiv_rn(hw, 2.0));
    r.aa = (long long)ceil(__ddiv_rn(__dsub_rn(beg, g.begin_wave), g.mask_step));
    r.bb = (long long)(ceil(__ddiv_rn(__dsub_rn(end, g.begin_wave), g.mask_step)) - 1);
    r.w = weight;
    r.ok = (r.aa - 1 >= 0) && (r.bb + 1 < g.n_ext) && (r.aa < g.n_ext) && (r.bb >= 0);
    r.frb = r.fra = 0.0;
    if (r.ok) {
        double wa = ccf_we(g, wt, r.aa), wa1 = ccf_we(g, wt, r.aa - 1);
        double wb = ccf_we(g, wt, r.bb), wb1 = ccf_we(g, wt, r.bb + 1);
        r.frb = __ddiv_rn(fabs(__dsub_rn(wa, beg)), __dsub_rn(wa, wa1));
        r.fra = __ddiv_rn(fabs(__dsub_rn(wb, end)), __dsub_rn(wb1, wb));
    }
    return r;
}

// pass 1: highest write sequence per (velocity, pixel of the slice);
// seq = 3*line + {0: hole interior, 1: pixel aa-1, 2: pixel bb}
__global__ void k_ccf_owner(CcfGeom g, const double *__restrict__ wt, const double *__restrict__ vel,
                            const double *__restrict__ lw, const double *__restrict__ lwt, int n_lines, int n_v,
                            int *owner, int *status) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n_lines * n_v) return;
    int iv = (int)(t / n_lines), l = (int)(t % n_lines);
    LineWin r = ccf_line(g, wt, vel[iv], lw[l], lwt[l]);
    if (!r.ok) { atomicExch(status, 11); return; }
    int *ow = owner + (long long)iv * g.n_w;
    for (long long k = r.aa; k < r.bb; ++k) {
        long long p = k - g.index_old;
        if (p >= 0 && p < g.n_w) atomicMax(&ow[p], 3 * l + 0);
    }
    long long p1 = r.aa - 1 - g.index_old, p2 = r.bb - g.index_old;
    if (p1 >= 0 && p1 < g.n_w) atomicMax(&ow[p1], 3 * l + 1);
    if (p2 >= 0 && p2 < g.n_w) atomicMax(&ow[p2], 3 * l + 2);
}

// pass 2: count the pixels each (velocity, line) owns
__global__ void k_ccf_count(CcfGeom g, const double *__restrict__ wt, const double *__restrict__ vel,
                            const double *__restrict__ lw, const double *__restrict__ lwt, int n_lines, int n_v,
                            const int *__restrict__ owner, int *cnt) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n_lines * n_v) return;
    int iv = (int)(t / n_lines), l = (int)(t % n_lines);
    LineWin r = ccf_line(g, wt, vel[iv], lw[l], lwt[l]);
    int c = 0;
    if (r.ok) {
        const int *ow = owner + (long long)iv * g.n_w;
        for (long long k = r.aa - 1; k <= r.bb; ++k) {
            long long p = k - g.index_old;
            if (p >= 0 && p < g.n_w && ow[p] >= 0 && ow[p] / 3 == l) ++c;
        }
    }
    cnt[t] = c;
}

// exclusive scan of counts per velocity row (one block per velocity)
__global__ void __launch_bounds__(1024) k_ccf_scan(int n_lines, const int *__restrict__ cnt, int *off, int *row_tot) {
    const int *c = cnt + (long long)blockIdx.x * n_lines;
    int *o = off + (long long)blockIdx.x * n_lines;
    __shared__ int warp_tot[32];
    __shared__ int base;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    for (int s = 0; s < n_lines; s += blockDim.x) {
        int i = s + threadIdx.x;
        int v = (i < n_lines) ? c[i] : 0;
        int x = v;
        for (int d = 1; d < 32; d <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) warp_tot[w] = x;
        __syncthreads();
        if (w == 0) {
            int t = (lane < nw) ? warp_tot[lane] : 0;
            for (int d = 1; d < 32; d <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, t, d);
                if (lane >= d) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        int pre = (w == 0 ? 0 : warp_tot[w - 1]) + x - v;
        if (i < n_lines) o[i] = base + pre;
        __syncthreads();
        if (threadIdx.x == 0) base += warp_tot[nw - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) row_tot[blockIdx.x] = base;
}

// pass 3: write the (pixel, value) entries of each velocity row
__global__ void k_ccf_fill(CcfGeom g, const double *__restrict__ wt, const double *__restrict__ vel,
                           const double *__restrict__ lw, const double *__restrict__ lwt, int n_lines, int n_v,
                           const int *__restrict__ owner, const int *__restrict__ off, long long row_cap,
                           int *col, double *val) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n_lines * n_v) return;
    int iv = (int)(t / n_lines), l = (int)(t % n_lines);
    LineWin r = ccf_line(g, wt, vel[iv], lw[l], lwt[l]);
    if (!r.ok) return;
    const int *ow = owner + (long long)iv * g.n_w;
    long long o = (long long)iv * row_cap + off[t];
    for (long long k = r.aa - 1; k <= r.bb; ++k) {
        long long p = k - g.index_old;
        if (p < 0 || p >= g.n_w) continue;
        int s = ow[p];
        if (s < 0 || s / 3 != l) continue;
        int kind = s % 3;
        double v = kind == 0 ? r.w : (kind == 1 ? __dmul_rn(r.w, r.frb) : __dmul_rn(r.w, r.fra));
        col[o] = (int)p;
        val[o] = v;
        ++o;
    }
}

// dot products: block (velocity, spectrum batch); FP64, or FP32 products with
// compensated FP32 partial sums assembled in FP64
template <bool F32, int SB>
__global__ void __launch_bounds__(256) k_ccf_dot(int n_w, const int *__restrict__ col, const double *__restrict__ val,
                                                 const int *__restrict__ row_tot, long long row_cap, int n_spec,
                                                 const double *__restrict__ spec, long long spec_stride,
                                                 double *ccf, int n_v) {
    int iv = blockIdx.x;
    int s0 = blockIdx.y * SB;
    int nsb = min(SB, n_spec - s0);
    int nnz = row_tot[iv];
    const int *c = col + (long long)iv * row_cap;
    const double *v = val + (long long)iv * row_cap;
    double acc[SB];
    float fs[SB], fc[SB];
#pragma unroll
    for (int q = 0; q < SB; ++q) { acc[q] = 0.0; fs[q] = 0.f; fc[q] = 0.f; }
    for (int k = threadIdx.x; k < nnz; k += blockDim.x) {
        int p = c[k];
        double w = v[k];
#pragma unroll
        for (int q = 0; q < SB; ++q) {
            if (q < nsb) {
                double x = spec[(long long)(s0 + q) * spec_stride + p];
                if (F32) {
                    float y = (float)w * (float)x - fc[q];
                    float t = fs[q] + y;
                    fc[q] = (t - fs[q]) - y;
                    fs[q] = t;
                } else {
                    acc[q] = fma(w, x, acc[q]);
                }
            }
        }
    }
    __shared__ double red[8][SB];
#pragma unroll
    for (int q = 0; q < SB; ++q) {
        double a = F32 ? ((double)fs[q] - (double)fc[q]) : acc[q];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][q] = a;
    }
    __syncthreads();
    if (threadIdx.x < SB && threadIdx.x < nsb) {
        double a = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a += red[w][threadIdx.x];
        ccf[(long long)(s0 + threadIdx.x) * n_v + iv] = a;
    }
}

// the apodisation window of run_all_SOAP.py:306-311 at velocity index i
__device__ __forceinline__ double ccf_apod(int i, int n_v) {
    const int nb_zeros = 5;
    const int period = (int)((n_v - 1) / 2.);
    const int len_app = (int)(period / 2.);
    const int n_ones = n_v - period - 2 * nb_zeros;
    if (i < nb_zeros) return 0.0;
    if (i < nb_zeros + len_app) {
        int a = i - nb_zeros;
        return 0.5 * cos(2 * SOAP_PI / period * a - SOAP_PI) + 0.5;
    }
    if (i < nb_zeros + len_app + n_ones) return 1.0;
    if (i < nb_zeros + 2 * len_app + n_ones) {
        int a = len_app - 1 - (i - nb_zeros - len_app - n_ones);
        return 0.5 * cos(2 * SOAP_PI / period * a - SOAP_PI) + 0.5;
    }
    return 0.0;
}

// normalise by the max and apodise, run_all_SOAP.py:299-314,369-370
__global__ void k_ccf_normalise(int n_spec, int n_v, double *ccf) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_spec) return;
    double *c = ccf + (long long)s * n_v;
    double mx = c[0];
    for (int i = 1; i < n_v; ++i) mx = fmax(mx, c[i]);
    for (int i = 0; i < n_v; ++i) {
        double v = c[i] / mx;
        c[i] = 1 - ((-v + 1) * ccf_apod(i, n_v));
    }
}

extern "C" int soapgb_ccf(soapgb_ctx *ctx, int form, int n_v, const double *vel, int n_lines,
                          const double *line_wave, const double *line_weight, int n_w, const double *wave_trim,
                          double step_size, double wave_extend, double mask_step, int index_old, int n_spec,
                          const double *spectra, int normalise, int mem, double *ccf_out) {
    if (!ctx) return SOAPGB_ERR_ARG;
    if (n_v < 1 || n_lines < 0 || n_w < 2 || n_spec < 0 || !vel || !wave_trim || !ccf_out ||
        (n_lines > 0 && (!line_wave || !line_weight)) || (n_spec > 0 && !spectra) || !(step_size > 0) ||
        !(mask_step > 0))
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_ccf: bad arguments");
    if (normalise) {
        int period = (int)((n_v - 1) / 2.), len_app = (int)(period / 2.);
        if (n_v < 21 || 2 * len_app != period)
            return set_error(ctx, SOAPGB_ERR_ARG,
                             "soapgb_ccf: the apodisation window of run_all_SOAP.py:306-311 needs "
                             "(n_v-1)/2 even and n_v >= 21 (n_v = %d)", n_v);
    }
    if (n_spec == 0) return SOAPGB_OK;
    SOAP_DEVICE(ctx);
    int np_ext = (int)(wave_extend / step_size);
    long long n_ext = (long long)n_w + 2LL * np_ext;
    if (n_ext - 2LL * index_old != n_w)
        return set_error(ctx, SOAPGB_ERR_ARG,
                         "soapgb_ccf: mask slice [%d:-%d] of the %lld-point extended grid does not give %d points",
                         index_old, index_old, n_ext, n_w);
    bool host = (mem == SOAPGB_HOST);
    double w_first, w_last;
    if (host) {
        w_first = wave_trim[0];
        w_last = wave_trim[n_w - 1];
    } else {
        SOAP_CUDA(ctx, cudaMemcpyAsync(&w_first, wave_trim, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(&w_last, wave_trim + n_w - 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    if (!(w_last > w_first)) return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_ccf: wavelengths must ascend");
    CcfGeom g;
    g.np_ext = np_ext;
    g.n_ext = (int)n_ext;
    g.n_w = n_w;
    g.index_old = index_old;
    g.mask_step = mask_step;
    g.start_b = w_first - step_size * np_ext;
    g.stop_b = w_first;
    g.start_a = w_last;
    g.stop_a = w_last + step_size * np_ext;
    g.begin_wave = std::min(g.start_b, w_first);
    double beta = 820. / SOAP_C_LIGHT;
    g.k_hw = sqrt((1 + beta) / (1 - beta)) - 1;
    long long nt = (long long)n_lines * n_v;
    // a (velocity, line) owns at most bb - aa + 2 pixels: bound it by the widest hole
    double hw_max = std::max(std::fabs(w_first), std::fabs(w_last) + wave_extend) * 1.001 * g.k_hw;
    long long per_line = (long long)ceil(hw_max / mask_step) + 3;
    long long row_cap = per_line * n_lines + 16;
    Workspace ws(ctx);
    int s_vel = ws.add(host ? sizeof(double) * n_v : 0);
    int s_lw = ws.add(host ? sizeof(double) * (n_lines > 0 ? n_lines : 1) : 0);
    int s_lwt = ws.add(host ? sizeof(double) * (n_lines > 0 ? n_lines : 1) : 0);
    int s_wt = ws.add(host ? sizeof(double) * n_w : 0);
    int s_spec = ws.add(host ? sizeof(double) * (size_t)n_w * n_spec : 0);
    int s_out = ws.add(host ? sizeof(double) * (size_t)n_v * n_spec : 0);
    int s_owner = ws.add(sizeof(int) * (size_t)n_w * n_v);
    int s_cnt = ws.add(sizeof(int) * (nt > 0 ? nt : 1));
    int s_off = ws.add(sizeof(int) * (nt > 0 ? nt : 1));
    int s_tot = ws.add(sizeof(int) * n_v);
    int s_col = ws.add(sizeof(int) * row_cap * n_v);
    int s_val = ws.add(sizeof(double) * row_cap * n_v);
    int rc = ws.commit();
    if (rc) return rc;
    const double *d_vel = (const double *)stage_in(ctx, mem, vel, sizeof(double) * n_v, ws.get<void>(s_vel), &rc);
    if (rc) return rc;
    const double *d_lw = (const double *)stage_in(ctx, mem, line_wave, sizeof(double) * n_lines, ws.get<void>(s_lw), &rc);
    if (rc) return rc;
    const double *d_lwt = (const double *)stage_in(ctx, mem, line_weight, sizeof(double) * n_lines, ws.get<void>(s_lwt), &rc);
    if (rc) return rc;
    const double *d_wt = (const double *)stage_in(ctx, mem, wave_trim, sizeof(double) * n_w, ws.get<void>(s_wt), &rc);
    if (rc) return rc;
    const double *d_spec = (const double *)stage_in(ctx, mem, spectra, sizeof(double) * (size_t)n_w * n_spec, ws.get<void>(s_spec), &rc);
    if (rc) return rc;
    double *d_out = host ? ws.get<double>(s_out) : ccf_out;
    int *owner = ws.get<int>(s_owner);
    int *cnt = ws.get<int>(s_cnt), *off = ws.get<int>(s_off), *tot = ws.get<int>(s_tot);
    int *col = ws.get<int>(s_col);
    double *val = ws.get<double>(s_val);
    SOAP_CUDA(ctx, cudaMemsetAsync(owner, 0xff, sizeof(int) * (size_t)n_w * n_v, ctx->stream));   // -1
    if (nt > 0) {
        int gb = grid_for(ctx, nt, 256);
        SOAP_TRACED(ctx, "ccf_mask", k_ccf_owner<<<gb, 256, 0, ctx->stream>>>(g, d_wt, d_vel, d_lw, d_lwt, n_lines, n_v, owner, ctx->d_status));
        SOAP_LAUNCHED(ctx);
        SOAP_TRACED(ctx, "ccf_mask", k_ccf_count<<<gb, 256, 0, ctx->stream>>>(g, d_wt, d_vel, d_lw, d_lwt, n_lines, n_v, owner, cnt));
        SOAP_LAUNCHED(ctx);
        SOAP_TRACED(ctx, "ccf_mask", k_ccf_scan<<<n_v, 1024, 0, ctx->stream>>>(n_lines, cnt, off, tot));
        SOAP_LAUNCHED(ctx);
        SOAP_TRACED(ctx, "ccf_mask", k_ccf_fill<<<gb, 256, 0, ctx->stream>>>(g, d_wt, d_vel, d_lw, d_lwt, n_lines, n_v, owner, off, row_cap,
                                                col, val));
        SOAP_LAUNCHED(ctx);
    } else {
        SOAP_CUDA(ctx, cudaMemsetAsync(tot, 0, sizeof(int) * n_v, ctx->stream));
    }
    if (form == SOAPGB_FAST32) {
        dim3 gd(n_v, (n_spec + 7) / 8);
        SOAP_TRACED(ctx, "ccf_dot", k_ccf_dot<true, 8><<<gd, 256, 0, ctx->stream>>>(n_w, col, val, tot, row_cap, n_spec, d_spec, n_w, d_out, n_v));
    } else {
        dim3 gd(n_v, (n_spec + 7) / 8);
        SOAP_TRACED(ctx, "ccf_dot", k_ccf_dot<false, 8><<<gd, 256, 0, ctx->stream>>>(n_w, col, val, tot, row_cap, n_spec, d_spec, n_w, d_out, n_v));
    }
    SOAP_LAUNCHED(ctx);
    if (normalise) {
        k_ccf_normalise<<<(n_spec + 63) / 64, 64, 0, ctx->stream>>>(n_spec, n_v, d_out);
        SOAP_LAUNCHED(ctx);
    }
    rc = check_status(ctx, "soapgb_ccf");
    if (rc) return set_error(ctx, rc, "soapgb_ccf: a mask hole reaches past the extended wavelength grid");
    if (host) {
        SOAP_CUDA(ctx, cudaMemcpyAsync(ccf_out, d_out, sizeof(double) * (size_t)n_v * n_spec, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return SOAPGB_OK;
}

// ---------------------------------------------------------------------------
// Adjoint of the CCF (the differentiable form; the reference has no gradient path).
// The raw CCF is linear in the spectra, ccf[s, v] = sum_p M[v, p] spec[s, p], so its
// adjoint is grad[s, p] = sum_v M[v, p] g[s, v].  Each (velocity, pixel) has one
// owner line in the mask (the forward's owner map), so one thread per pixel walks
// the velocities in order and recomputes its mask value: no transpose, no atomics.
// The normalisation out_i = 1 - (1 - c_i / mx) app_i (mx the max, first index at
// ties) contributes dL/dc_i = app_i G_i / mx - [i = i_mx] sum_j G_j app_j c_j / mx^2.
// ---------------------------------------------------------------------------
__global__ void k_ccf_norm_adj(int n_spec, int n_v, const double *__restrict__ raw, const double *__restrict__ g,
                               double *__restrict__ gc) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_spec) return;
    const double *c = raw + (long long)s * n_v;
    const double *gs = g + (long long)s * n_v;
    double *o = gc + (long long)s * n_v;
    double mx = c[0];
    int imx = 0;
    for (int i = 1; i < n_v; ++i)
        if (c[i] > mx) { mx = c[i]; imx = i; }
    double S = 0.0;
    for (int i = 0; i < n_v; ++i) {
        const double app = ccf_apod(i, n_v);
        S = fma(gs[i] * app, c[i], S);
        o[i] = app * gs[i] / mx;
    }
    o[imx] -= S / (mx * mx);
}

template <int SB>
__global__ void __launch_bounds__(256) k_ccf_adj(CcfGeom g, const double *__restrict__ wt,
                                                 const double *__restrict__ vel, const double *__restrict__ lw,
                                                 const double *__restrict__ lwt, int n_v,
                                                 const int *__restrict__ owner, int n_spec,
                                                 const double *__restrict__ gc, double *__restrict__ grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= g.n_w) return;
    const int s0 = blockIdx.y * SB;
    const int nsb = min(SB, n_spec - s0);
    double acc[SB];
#pragma unroll
    for (int q = 0; q < SB; ++q) acc[q] = 0.0;
    for (int iv = 0; iv < n_v; ++iv) {
        const int sq = owner[(long long)iv * g.n_w + p];
        if (sq < 0) continue;
        const int l = sq / 3, kind = sq % 3;
        const LineWin r = ccf_line(g, wt, vel[iv], lw[l], lwt[l]);
        const double m = kind == 0 ? r.w : (kind == 1 ? __dmul_rn(r.w, r.frb) : __dmul_rn(r.w, r.fra));
#pragma unroll
        for (int q = 0; q < SB; ++q)
            if (q < nsb) acc[q] = fma(m, gc[(long long)(s0 + q) * n_v + iv], acc[q]);
    }
#pragma unroll
    for (int q = 0; q < SB; ++q)
        if (q < nsb) grad[(long long)(s0 + q) * g.n_w + p] = acc[q];
}

extern "C" int soapgb_ccf_adjoint(soapgb_ctx *ctx, int n_v, const double *vel, int n_lines,
                                  const double *line_wave, const double *line_weight, int n_w,
                                  const double *wave_trim, double step_size, double wave_extend, double mask_step,
                                  int index_old, int n_spec, const double *ccf_raw, int normalise,
                                  const double *g_ccf, int mem, double *grad_spectra) {
    if (!ctx) return SOAPGB_ERR_ARG;
    if (n_v < 1 || n_lines < 0 || n_w < 2 || n_spec < 0 || !vel || !wave_trim || !g_ccf || !grad_spectra ||
        (n_lines > 0 && (!line_wave || !line_weight)) || (normalise && n_spec > 0 && !ccf_raw) ||
        !(step_size > 0) || !(mask_step > 0))
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_ccf_adjoint: bad arguments");
    if (normalise) {
        // the forward's apodisation window (run_all_SOAP.py:306-311) exists only for these n_v
        int period = (int)((n_v - 1) / 2.), len_app = (int)(period / 2.);
        if (n_v < 21 || 2 * len_app != period)
            return set_error(ctx, SOAPGB_ERR_ARG,
                             "soapgb_ccf_adjoint: the apodisation window of run_all_SOAP.py:306-311 needs "
                             "(n_v-1)/2 even and n_v >= 21 (n_v = %d)", n_v);
    }
    if (n_spec == 0) return SOAPGB_OK;
    SOAP_DEVICE(ctx);
    const int np_ext = (int)(wave_extend / step_size);
    const long long n_ext = (long long)n_w + 2LL * np_ext;
    if (n_ext - 2LL * index_old != n_w)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_ccf_adjoint: mask slice does not give %d points", n_w);
    const bool host = (mem == SOAPGB_HOST);
    double w_first, w_last;
    if (host) {
        w_first = wave_trim[0];
        w_last = wave_trim[n_w - 1];
    } else {
        SOAP_CUDA(ctx, cudaMemcpyAsync(&w_first, wave_trim, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(&w_last, wave_trim + n_w - 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    if (!(w_last > w_first)) return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_ccf_adjoint: wavelengths must ascend");
    CcfGeom g;
    g.np_ext = np_ext;
    g.n_ext = (int)n_ext;
    g.n_w = n_w;
    g.index_old = index_old;
    g.mask_step = mask_step;
    g.start_b = w_first - step_size * np_ext;
    g.stop_b = w_first;
    g.start_a = w_last;
    g.stop_a = w_last + step_size * np_ext;
    g.begin_wave = std::min(g.start_b, w_first);
    const double beta = 820. / SOAP_C_LIGHT;
    g.k_hw = sqrt((1 + beta) / (1 - beta)) - 1;
    const long long nt = (long long)n_lines * n_v;
    const size_t vs_b = sizeof(double) * (size_t)n_v * n_spec, ws_b = sizeof(double) * (size_t)n_w * n_spec;
    Workspace ws(ctx);
    int s_vel = ws.add(host ? sizeof(double) * n_v : 0);
    int s_lw = ws.add(host ? sizeof(double) * (n_lines > 0 ? n_lines : 1) : 0);
    int s_lwt = ws.add(host ? sizeof(double) * (n_lines > 0 ? n_lines : 1) : 0);
    int s_wt = ws.add(host ? sizeof(double) * n_w : 0);
    int s_raw = ws.add(host && normalise ? vs_b : 0);
    int s_g = ws.add(host ? vs_b : 0);
    int s_out = ws.add(host ? ws_b : 0);
    int s_gc = ws.add(normalise ? vs_b : 0);
    int s_owner = ws.add(sizeof(int) * (size_t)n_w * n_v);
    int rc = ws.commit();
    if (rc) return rc;
#define STAGE(dst, src, bytes, slot)                                                  \
    dst = (const double *)stage_in(ctx, mem, src, bytes, ws.get<void>(slot), &rc);   \
    if (rc) return rc;
    const double *d_vel, *d_lw, *d_lwt, *d_wt, *d_raw, *d_g;
    STAGE(d_vel, vel, sizeof(double) * n_v, s_vel);
    STAGE(d_lw, line_wave, sizeof(double) * n_lines, s_lw);
    STAGE(d_lwt, line_weight, sizeof(double) * n_lines, s_lwt);
    STAGE(d_wt, wave_trim, sizeof(double) * n_w, s_wt);
    STAGE(d_raw, normalise ? ccf_raw : nullptr, normalise ? vs_b : 0, s_raw);
    STAGE(d_g, g_ccf, vs_b, s_g);
#undef STAGE
    double *d_out = host ? ws.get<double>(s_out) : grad_spectra;
    int *owner = ws.get<int>(s_owner);
    SOAP_CUDA(ctx, cudaMemsetAsync(owner, 0xff, sizeof(int) * (size_t)n_w * n_v, ctx->stream));   // -1
    if (nt > 0) {
        k_ccf_owner<<<grid_for(ctx, nt, 256), 256, 0, ctx->stream>>>(g, d_wt, d_vel, d_lw, d_lwt, n_lines, n_v, owner,
                                                                     ctx->d_status);
        SOAP_LAUNCHED(ctx);
    }
    const double *gc = d_g;
    if (normalise) {
        double *t = ws.get<double>(s_gc);
        k_ccf_norm_adj<<<(n_spec + 63) / 64, 64, 0, ctx->stream>>>(n_spec, n_v, d_raw, d_g, t);
        SOAP_LAUNCHED(ctx);
        gc = t;
    }
    SOAP_TRACED(ctx, "ccf_adjoint",
                (k_ccf_adj<8><<<dim3(grid_for(ctx, n_w, 256), (n_spec + 7) / 8), 256, 0, ctx->stream>>>(
                    g, d_wt, d_vel, d_lw, d_lwt, n_v, owner, n_spec, gc, d_out)));
    SOAP_LAUNCHED(ctx);
    rc = check_status(ctx, "soapgb_ccf_adjoint");
    if (rc) return set_error(ctx, rc, "soapgb_ccf_adjoint: a mask hole reaches past the extended wavelength grid");
    if (host) {
        SOAP_CUDA(ctx, cudaMemcpyAsync(grad_spectra, d_out, ws_b, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return SOAPGB_OK;
}
