// a8 / a14: instrumental Gaussian convolution, min/max reductions, normalisation.
//
// Reference: SOAP_initialize.cu:69-96,206-294,437-505 and SOAP_resolution.cu:66-310
// (wav_sigma, conv_inst, reduceMax/MinIdxOptimizedShared, spec_diff, spec_norm:
// six launches and four blocking copies per spectrum, every reduction block
// scanning the whole array).  Here:
//   PLAIN64  -- conv_inst's arithmetic term by term (one thread per pixel, all
//               2w-1 taps, the reference's operation order), batched over spectra;
//   FAST64 / FAST32 -- the convolution is linear, so
//               C = conv(1 - base) + conv(spec);
//               conv(1 - base) is computed once per base in FP64 and the per-phase
//               part conv(spec) uses shared tap weights (FP64, or FP32 with FP64
//               assembly), register-blocked four pixels per thread over staged
//               spectrum windows.  Taps whose weight is below e^-40 (FAST64) or
//               e^-30 (FAST32) of the central one are skipped.
//   min / max -- one pass per spectrum with order-preserving 64-bit integer atomics
//               (deterministic), then an FP64 normalisation pass.
#include <algorithm>
#include <cmath>
#include <climits>
#include <vector>

#include "internal.cuh"
#include "resolution.cuh"

using namespace soapgb;

// Delta_lambda_cpu, SOAP_initialize.cu:39-50 (float sqrtf on a double argument)
static double host_delta_lambda_f32(double line_width, double lambda_line0) {
    double beta = line_width / SOAP_C_LIGHT;
    return -1 * lambda_line0 * (1 - (double)sqrtf((float)((1 + beta) / (1 - beta))));
}

// rndup, SOAP_initialize.cu:19-36
static double host_rndup(double n, int nb_decimal) {
    double t = n * pow(10, nb_decimal) - floor(n * pow(10, nb_decimal));
    if (t >= 0.5) {
        n *= pow(10, nb_decimal);
        n = ceil(n);
        n /= pow(10, nb_decimal);
    } else {
        n *= pow(10, nb_decimal);
        n = floor(n);
        n /= pow(10, nb_decimal);
    }
    return n;
}

// Delta_lambda(sigma_v, lambda) / lambda (SOAP_initialize.cu:55-66 without the factor lambda)
static double soap_sigma_per_lambda(double sigma_v) {
    double beta = sigma_v / SOAP_C_LIGHT;
    return -1 * (1 - sqrt((1 + beta) / (1 - beta)));
}

namespace soapgb {
int conv_halfwidth(double wave0, double wave1, double sigma_v, double window) {
    double wavelength_step = wave1 - wave0;
    return (int)host_rndup((window * host_delta_lambda_f32(sigma_v, wave0)) / wavelength_step, 0);
}
}  // namespace soapgb

__device__ __forceinline__ unsigned long long soap_ord_enc(double v) { return soap_ord64(v); }
__device__ __forceinline__ double soap_ord_dec(unsigned long long u) {
    u = (u & 0x8000000000000000ULL) ? (u & 0x7fffffffffffffffULL) : ~u;
    return __longlong_as_double((long long)u);
}

// spectrum s uses base_b when b_every > 0 and s % b_every == b_every - 1
__device__ __forceinline__ const double *soap_base_for(int s, const double *base_a, const double *base_b, int b_every) {
    if (b_every > 0 && (s % b_every) == b_every - 1) return base_b;
    return base_a;
}

// ---------------------------------------------------------------------------
// PLAIN64 convolution: conv_inst term by term.  grid (pixel blocks, spectra)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_conv_plain64(int n, int n_eff, const double *__restrict__ lam,
                                                      const double *__restrict__ spec, long long spec_stride,
                                                      const double *__restrict__ base_a,
                                                      const double *__restrict__ base_b, int b_every,
                                                      double sigma_v, int wid, double step_mult, double step_exp,
                                                      double *__restrict__ conv, long long conv_stride) {
    int s = blockIdx.y;
    int index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= n_eff) return;
    const double *sp = spec + (long long)s * spec_stride;
    const double *bp = soap_base_for(s, base_a, base_b, b_every);
    double acc = 0.0;
    if ((index > wid) && (index + wid < n - 1)) {
        double sig = soap_delta_lambda(sigma_v, lam[index]);
        double norm = __dmul_rn(sig, sqrt(2. * SOAP_PI));
        double den = __dmul_rn(__dmul_rn(2.0, sig), sig);
        for (int m = index - wid; m < index + wid - 1; m++) {
            int d = m - index;
            double a = bp ? __dsub_rn(bp[m], sp[m]) : sp[m];
            double e = exp(__ddiv_rn(__dmul_rn(__dmul_rn((double)(-d * d), step_exp), step_exp), den));
            double t = __dmul_rn(__ddiv_rn(__dmul_rn(__dmul_rn(step_mult, __dsub_rn(1.0, a)), 1.), norm), e);
            acc = __dadd_rn(acc, t);
        }
    }
    conv[(long long)s * conv_stride + index] = acc;
}

// per-pixel tap parameters of the fast forms: weight scale kq = step_mult / (s sqrt(2 pi)),
// exponent coefficient cq = step_exp^2 / (2 s^2), significant tap range [dlo, dhi]
// (dhi < dlo marks a pixel outside the reference's convolution interior)
template <typename T>
__global__ void k_conv_params(int n, int n_eff, const double *__restrict__ lam, double ka, double kb, double kr,
                              int wid, int halo, T *kq, T *cq, int2 *rng) {
    // sigma_i = lambda_i (sqrt((1 + b)/(1 - b)) - 1) is proportional to lambda_i, so with
    // ka = step_mult / (s1 sqrt(2 pi)), kb = step_exp^2 / (2 s1^2), kr = sqrt(cut / kb)
    // (s1 = sigma at lambda = 1): kq = ka / lambda, cq = kb / lambda^2, reach = kr lambda
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_eff) return;
    bool live = (i > wid) && (i + wid < n - 1);
    double k = 0.0, c = 0.0;
    int lo = 0, hi = -1;
    if (live) {
        const double l = lam[i];
        const double inv = 1.0 / l;
        k = ka * inv;
        c = kb * inv * inv;
        int r = (int)floor(kr * l);
        lo = max(max(-wid, -r), -halo);
        hi = min(min(wid - 2, r), halo);
    }
    kq[i] = (T)k;
    cq[i] = (T)c;
    rng[i] = make_int2(lo, hi);
}

// ---------------------------------------------------------------------------
// FAST convolution of x (no "1 -"): out[i] = sum_d w_i(d) x[i+d], d in the
// reference window [-wid, wid-2] intersected with the significant taps.  Block =
// 256 threads x 4 pixels = 1024 pixels; SB spectra per block staged in smem.
// sign: +1 for conv(x), or the base pass computes conv(1 - base) with x = 1 - base.
// ---------------------------------------------------------------------------
constexpr int FC_THREADS = 256;
constexpr int FC_PIX = 4;
constexpr int FC_TILE = FC_THREADS * FC_PIX;

template <typename T, int SB, typename SrcT, typename OutT>
__global__ void __launch_bounds__(FC_THREADS) k_conv_fast(int n, int n_eff, const T *__restrict__ kqa,
                                                          const T *__restrict__ cqa, const int2 *__restrict__ rnga,
                                                          const SrcT *__restrict__ spec, long long spec_stride,
                                                          int n_spec, int one_minus, int halo,
                                                          OutT *__restrict__ conv, long long conv_stride) {
    extern __shared__ unsigned char smem_raw[];
    T *xs = reinterpret_cast<T *>(smem_raw);
    int win = FC_TILE + 2 * halo;
    int i0 = blockIdx.x * FC_TILE;
    int s0 = blockIdx.y * SB;
    int nsb = min(SB, n_spec - s0);
    // stage [i0 - halo, i0 + FC_TILE + halo) of each spectrum (0 outside [0, n))
    for (int q = 0; q < nsb; ++q) {
        const SrcT *sp = spec + (long long)(s0 + q) * spec_stride;
        for (int t = threadIdx.x; t < win; t += FC_THREADS) {
            int m = i0 - halo + t;
            T v = (m >= 0 && m < n) ? (T)sp[m] : (T)0;
            if (one_minus) v = (m >= 0 && m < n) ? (T)1 - v : (T)0;
            xs[q * win + t] = v;
        }
    }
    __syncthreads();
    int ib = i0 + threadIdx.x * FC_PIX;   // first pixel of this thread
    T acc[SB][FC_PIX];
#pragma unroll
    for (int q = 0; q < SB; ++q)
#pragma unroll
        for (int p = 0; p < FC_PIX; ++p) acc[q][p] = (T)0;
    T kq[FC_PIX], cq[FC_PIX];
    int dlo[FC_PIX], dhi[FC_PIX];
    int elo = 1 << 30, ehi = -(1 << 30);
#pragma unroll
    for (int p = 0; p < FC_PIX; ++p) {
        int i = ib + p;
        kq[p] = (T)0;
        cq[p] = (T)0;
        dlo[p] = 0;
        dhi[p] = -1;
        if (i < n_eff) {
            kq[p] = kqa[i];
            cq[p] = cqa[i];
            int2 r = rnga[i];
            dlo[p] = r.x;
            dhi[p] = r.y;
            if (r.x <= r.y) {
                elo = min(elo, i + r.x);
                ehi = max(ehi, i + r.y);
            }
        }
    }
    // FP64: Gaussian weights by the exact-product recurrence exp(-(d+1)^2 c) =
    // exp(-d^2 c) exp(-(2d+1) c), exp(-(2d+3) c) = exp(-(2d+1) c) exp(-2c): three exp per
    // pixel instead of one per tap (rounding grows by ~1e-16 per tap).  FP32: one
    // MUFU exp per tap.
    T wcur[FC_PIX], rcur[FC_PIX], e2[FC_PIX];
    if constexpr (sizeof(T) == 8) {
#pragma unroll
        for (int p = 0; p < FC_PIX; ++p) {
            double c = cq[p], d0 = (double)dlo[p];
            wcur[p] = kq[p] * exp(-d0 * d0 * c);
            rcur[p] = exp(-(2.0 * d0 + 1.0) * c);
            e2[p] = exp(-2.0 * c);
        }
    }
    if (elo <= ehi) {
        for (int e = elo; e <= ehi; ++e) {
            T w[FC_PIX];
#pragma unroll
            for (int p = 0; p < FC_PIX; ++p) {
                int d = e - (ib + p);
                if (d >= dlo[p] && d <= dhi[p]) {
                    if constexpr (sizeof(T) == 4) {
                        w[p] = kq[p] * __expf(-(T)(d * d) * cq[p]);
                    } else {
                        w[p] = wcur[p];
                        wcur[p] *= rcur[p];
                        rcur[p] *= e2[p];
                    }
                } else {
                    w[p] = (T)0;
                }
            }
            int li = e - (i0 - halo);
#pragma unroll
            for (int q = 0; q < SB; ++q) {
                if (q < nsb) {
                    T xv = xs[q * win + li];
#pragma unroll
                    for (int p = 0; p < FC_PIX; ++p) acc[q][p] += w[p] * xv;
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < SB; ++q) {
        if (q >= nsb) continue;
        OutT *cp = conv + (long long)(s0 + q) * conv_stride;
#pragma unroll
        for (int p = 0; p < FC_PIX; ++p) {
            int i = ib + p;
            if (i < n_eff) cp[i] = (dlo[p] <= dhi[p]) ? (OutT)acc[q][p] : (OutT)0;
        }
    }
}

// --- the base convolution in double-float arithmetic on the FP32 pipe -------------------
// A value is the unevaluated sum hi + lo of two floats (about 48 significant bits).
// Products and sums use the error-free transforms of the published double-float
// arithmetic: TwoProduct through FMA (the rounding error of a * b is fma(a, b, -a*b))
// and Knuth's TwoSum, each followed by a renormalisation.
struct DFloat {
    float hi, lo;
};
__device__ __forceinline__ DFloat df_of(double v) {
    const float h = (float)v;
    return {h, (float)(v - (double)h)};
}
__device__ __forceinline__ DFloat df_renorm(float s, float e) {
    const float h = s + e;
    return {h, e - (h - s)};
}
__device__ __forceinline__ DFloat df_mul(DFloat a, DFloat b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return df_renorm(p, e);
}
__device__ __forceinline__ DFloat df_add(DFloat a, DFloat b) {
    const float s = a.hi + b.hi;
    const float bv = s - a.hi;
    float e = (a.hi - (s - bv)) + (b.hi - bv);
    e += a.lo + b.lo;
    return df_renorm(s, e);
}

// k_conv_fast's FP64 form (Gaussian weights by the exact-product recurrence, the same
// per-pixel ranges, conv(1 - base)) in double-float: the base convolution of the FP32
// form without FP64 arithmetic in the tap loop (the FP64 pipe is 1/64 of the FP32 one,
// and the kernel runs beside the FP64 geometry stages).  Results agree with the FP64
// form to about 1e-13 relative.  grid (tiles of 1024 px, bases / SB).
template <int SB>
__global__ void __launch_bounds__(FC_THREADS) k_conv_base_df(int n, int n_eff, const double *__restrict__ kqa,
                                                             const double *__restrict__ cqa,
                                                             const int2 *__restrict__ rnga,
                                                             const double *__restrict__ spec, long long spec_stride,
                                                             int n_spec, int halo, double *__restrict__ conv,
                                                             long long conv_stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *xs = reinterpret_cast<float2 *>(smem_raw);   // staged 1 - base as (hi, lo)
    const int win = FC_TILE + 2 * halo;
    const int i0 = blockIdx.x * FC_TILE;
    const int s0 = blockIdx.y * SB;
    const int nsb = min(SB, n_spec - s0);
    for (int q = 0; q < nsb; ++q) {
        const double *sp = spec + (long long)(s0 + q) * spec_stride;
        for (int t = threadIdx.x; t < win; t += FC_THREADS) {
            const int m = i0 - halo + t;
            const DFloat d = df_of((m >= 0 && m < n) ? 1.0 - sp[m] : 0.0);
            xs[q * win + t] = make_float2(d.hi, d.lo);
        }
    }
    __syncthreads();
    const int ib = i0 + threadIdx.x * FC_PIX;
    DFloat acc[SB][FC_PIX];
#pragma unroll
    for (int q = 0; q < SB; ++q)
#pragma unroll
        for (int p = 0; p < FC_PIX; ++p) acc[q][p] = {0.f, 0.f};
    DFloat wcur[FC_PIX], rcur[FC_PIX], e2[FC_PIX];
    int dlo[FC_PIX], dhi[FC_PIX];
    int elo = 1 << 30, ehi = -(1 << 30);
#pragma unroll
    for (int p = 0; p < FC_PIX; ++p) {
        const int i = ib + p;
        dlo[p] = 0;
        dhi[p] = -1;
        wcur[p] = rcur[p] = e2[p] = {0.f, 0.f};
        if (i < n_eff) {
            const int2 r = rnga[i];
            dlo[p] = r.x;
            dhi[p] = r.y;
            if (r.x <= r.y) {
                elo = min(elo, i + r.x);
                ehi = max(ehi, i + r.y);
                const double c = cqa[i], d0 = (double)r.x;
                wcur[p] = df_of(kqa[i] * exp(-d0 * d0 * c));
                rcur[p] = df_of(exp(-(2.0 * d0 + 1.0) * c));
                e2[p] = df_of(exp(-2.0 * c));
            }
        }
    }
    for (int e = elo; e <= ehi; ++e) {
        DFloat w[FC_PIX];
#pragma unroll
        for (int p = 0; p < FC_PIX; ++p) {
            const int d = e - (ib + p);
            if (d >= dlo[p] && d <= dhi[p]) {
                w[p] = wcur[p];
                wcur[p] = df_mul(wcur[p], rcur[p]);
                rcur[p] = df_mul(rcur[p], e2[p]);
            } else {
                w[p] = {0.f, 0.f};
            }
        }
        const int li = e - (i0 - halo);
#pragma unroll
        for (int q = 0; q < SB; ++q) {
            if (q < nsb) {
                const float2 xv = xs[q * win + li];
                const DFloat x = {xv.x, xv.y};
#pragma unroll
                for (int p = 0; p < FC_PIX; ++p) acc[q][p] = df_add(acc[q][p], df_mul(w[p], x));
            }
        }
    }
#pragma unroll
    for (int q = 0; q < SB; ++q) {
        if (q >= nsb) continue;
        double *cp = conv + (long long)(s0 + q) * conv_stride;
#pragma unroll
        for (int p = 0; p < FC_PIX; ++p) {
            const int i = ib + p;
            if (i < n_eff) cp[i] = (dlo[p] <= dhi[p]) ? (double)acc[q][p].hi + (double)acc[q][p].lo : 0.0;
        }
    }
}

// C_s += Cbase (FP64) where the reference has a C value; fused with min/max.
// grid (blocks, spectra).  A_s = base - spec over [0, n); C over [0, n_eff).
__global__ void __launch_bounds__(256) k_minmax(int n, int n_eff, const double *__restrict__ spec,
                                                long long spec_stride, const double *__restrict__ base_a,
                                                const double *__restrict__ base_b, int b_every,
                                                double *__restrict__ conv, long long conv_stride,
                                                const double *__restrict__ cb_a, const double *__restrict__ cb_b,
                                                unsigned long long *mm /* n_spec x 2: min A, max C */) {
    int s = blockIdx.y;
    const double *sp = spec + (long long)s * spec_stride;
    const double *bp = soap_base_for(s, base_a, base_b, b_every);
    const double *cb = soap_base_for(s, cb_a, cb_b, b_every);
    double *cp = conv + (long long)s * conv_stride;
    unsigned long long mn = ~0ULL, mx = 0ULL;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double a = bp ? __dsub_rn(bp[i], sp[i]) : sp[i];
        if (a == a) mn = min(mn, soap_ord_enc(a));
        if (i < n_eff) {
            double c = cp[i];
            if (cb) {   // fast forms: C = conv(1 - base) + conv(spec)
                c = __dadd_rn(cb[i], c);
                cp[i] = c;
            }
            if (c != 0.0 && c == c) mx = max(mx, soap_ord_enc(c));
        }
    }
    // block reduce
    __shared__ unsigned long long smn[8], smx[8];
    for (int o = 16; o > 0; o >>= 1) {
        mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { smn[w] = mn; smx[w] = mx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) { mn = min(mn, smn[q]); mx = max(mx, smx[q]); }
        atomicMin(&mm[2 * s], mn);
        if (mx != 0ULL) atomicMax(&mm[2 * s + 1], mx);
    }
}

__global__ void k_minmax_init(int n_spec, double sentinel, unsigned long long *mm) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n_spec) {
        mm[2 * s] = ~0ULL;
        mm[2 * s + 1] = soap_ord_enc(sentinel);
    }
}

// spec_norm: out = 1 - C (1 - min) / max
__global__ void __launch_bounds__(256) k_norm(int n_eff, const double *__restrict__ conv, long long conv_stride,
                                              const unsigned long long *__restrict__ mm, double *__restrict__ out,
                                              long long out_stride, double *minmax_out, int exact) {
    int s = blockIdx.y;
    double mn = soap_ord_dec(mm[2 * s]);
    double mx = soap_ord_dec(mm[2 * s + 1]);
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_eff) {
        double c = conv[(long long)s * conv_stride + i];
        if (exact)   // spec_norm's operation order (one division per pixel)
            out[(long long)s * out_stride + i] = __dsub_rn(1.0, __ddiv_rn(__dmul_rn(c, __dsub_rn(1.0, mn)), mx));
        else         // fast forms: one factor per spectrum
            out[(long long)s * out_stride + i] = 1.0 - c * ((1.0 - mn) / mx);
    }
    if (minmax_out && blockIdx.x == 0 && threadIdx.x == 0) {
        minmax_out[2 * s] = mn;
        minmax_out[2 * s + 1] = mx;
    }
}


// ---------------------------------------------------------------------------
// FAST32 reductions and normalisation.  The per-pixel work stays on the FP32
// pipe; the normalisation constants min A and max C are still exact FP64 values:
// pass 1 finds the FP32 extrema and, per block, the block's own extrema; pass 2
// re-evaluates in FP64 only the pixels of the blocks that can hold the exact
// extremum (FP32 value within 2^-21 of the magnitudes involved).
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned soap_ord32(float v) {
    unsigned u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float soap_dec32(unsigned u) {
    u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    return __uint_as_float(u);
}

__global__ void k_base_prep(int n, int n_eff, const double *__restrict__ base, const double *__restrict__ cb,
                            float *base32, float *cb32) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) base32[i] = (float)base[i];
    if (i < n_eff) cb32[i] = (float)cb[i];
}

__global__ void k_mm32_init(int n_spec, double sentinel, unsigned *mm32, unsigned long long *mm64) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n_spec) {
        if (mm32) {
            mm32[4 * s + 0] = 0xffffffffu;             // min A (FP32 key)
            mm32[4 * s + 1] = 0u;                      // max C (FP32 key)
            mm32[4 * s + 2] = 0u;                      // max(|base| + |spec|)
            mm32[4 * s + 3] = 0u;                      // max(|cb| + |conv|)
        }
        mm64[2 * s + 0] = ~0ULL;
        mm64[2 * s + 1] = soap_ord_enc(sentinel);
    }
}

// per-pixel tap constants of the FP32 convolution: weight(d) = 2^(d^2 c2 + lk) with
// c2 = -step_exp^2 / (2 s^2) log2(e), lk = log2(step_mult / (s sqrt(2 pi))) (FP64, then
// rounded once); live = inside the reference's convolution interior; rblk[b] = largest
// significant reach (weight >= e^-cut of the central one) over block b's pixels
__global__ void k_conv32_params(int n, int n_eff, const double *__restrict__ lam, double sigma_v, int wid, int halo,
                                double step_mult, double step_exp, double cut, float *c2, float *lk, int *live,
                                int *rblk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int reach = 0;
    if (i < n_eff) {
        bool lv = (i > wid) && (i + wid < n - 1);
        double a = 0.0, l = -200.0;
        if (lv) {
            double sig = soap_delta_lambda(sigma_v, lam[i]);
            double cq = step_exp * step_exp / (2.0 * sig * sig);
            a = -cq * 1.4426950408889634;   // log2(e)
            l = log2(step_mult / (sig * sqrt(2. * SOAP_PI)));
            reach = min((int)floor(sqrt(cut / cq)) + 1, halo);
        }
        c2[i] = (float)a;
        lk[i] = (float)l;
        live[i] = lv ? 1 : 0;
    }
    // a warp's pixels share one block of 1024: one atomic per warp
    reach = __reduce_max_sync(0xffffffffu, reach);
    if ((threadIdx.x & 31) == 0 && reach > 0) atomicMax(&rblk[(blockIdx.x * blockDim.x) / FC_TILE], reach);
}

// the FP32 tap constants from the FP64 ones of the base convolution (same pixels,
// same sigma): c2 = -cq log2(e), lk = log2(kq) (FP32 log2 of the rounded scale: one
// more rounding of the weights' scale), reach from the FP32 cut
__global__ void k_conv32_derive(int n_eff, const double *__restrict__ kq, const double *__restrict__ cq,
                                const int2 *__restrict__ rng, int halo, float cut, float *c2, float *lk, int *live,
                                int *rblk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int reach = 0;
    if (i < n_eff) {
        const int2 r = rng[i];
        const bool lv = r.x <= r.y;
        float a = 0.f, l = -200.f;
        if (lv) {
            const double c = cq[i];
            a = (float)(-c * 1.4426950408889634);
            l = log2f((float)kq[i]);
            reach = min((int)floorf(sqrtf(cut / (float)c)) + 1, halo);
        }
        c2[i] = a;
        lk[i] = l;
        live[i] = lv ? 1 : 0;
    }
    // a warp's pixels share one block of 1024: one atomic per warp
    reach = __reduce_max_sync(0xffffffffu, reach);
    if ((threadIdx.x & 31) == 0 && reach > 0) atomicMax(&rblk[(blockIdx.x * blockDim.x) / FC_TILE], reach);
}

__device__ __forceinline__ float soap_ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// --- FAST32 convolution, shared pieces -------------------------------------------------
// taps of 4 consecutive pixels ib .. ib+3 over SB staged spectra: xrow(q) + x0 is the
// staged value of source pixel ib - R - sh (x0 + 4 k is 16-byte aligned), R the block's
// reach, sh in [0, 3] the alignment shift; every weight one ex2.  The arithmetic runs on
// packed pairs over the pixel pairs (0, 1) and (2, 3): their exponents, and their sums,
// each staged value feeding two packed FMAs (one per pixel pair) in the scalar form's
// order, so the sums are the scalar FMA chain's bit for bit.
template <int SB>
__device__ __forceinline__ void conv32_taps(const float *xs, int win, int x0, int R, int sh, int wid,
                                            const float (&c2)[FC_PIX], const float (&lk)[FC_PIX],
                                            float (&acc)[SB][FC_PIX]) {
    // |d| <= R + 6 over the thread's taps: mask only if that can leave [-wid, wid - 2]
    const bool mask = (R + 8 > wid);
    const int nch = (3 + 2 * R + sh) / 4 + 1;
    // tap offset of tap 0 of the chunk at pixels (0, 1) and (2, 3), as pairs
    float e0 = (float)(-R - sh), e1 = e0 - 1.f, e2 = e0 - 2.f, e3 = e0 - 3.f;
    for (int ch = 0; ch < nch; ++ch) {
        float w[4][FC_PIX];   // w[k][p]: tap k of pixel p
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float da = e0, db = e1, dc = e2, dd = e3;
            soap_add2(da, db, (float)k, (float)k);
            soap_add2(dc, dd, (float)k, (float)k);
            float ya = lk[0], yb = lk[1], yc = lk[2], yd = lk[3], sa, sb, sc, sd;
            soap_mul2(sa, sb, da, db, da, db);
            soap_mul2(sc, sd, dc, dd, dc, dd);
            soap_fma2(ya, yb, sa, sb, c2[0], c2[1]);
            soap_fma2(yc, yd, sc, sd, c2[2], c2[3]);
            w[k][0] = soap_ex2(ya);
            w[k][1] = soap_ex2(yb);
            w[k][2] = soap_ex2(yc);
            w[k][3] = soap_ex2(yd);
            if (mask) {
                const float lo = (float)-wid, hi = (float)(wid - 2);
                if (da < lo || da > hi) w[k][0] = 0.f;
                if (db < lo || db > hi) w[k][1] = 0.f;
                if (dc < lo || dc > hi) w[k][2] = 0.f;
                if (dd < lo || dd > hi) w[k][3] = 0.f;
            }
        }
        soap_add2(e0, e1, 4.f, 4.f);
        soap_add2(e2, e3, 4.f, 4.f);
        const int li = x0 + 4 * ch;
#pragma unroll
        for (int q = 0; q < SB; ++q) {
            const float4 x4 = *reinterpret_cast<const float4 *>(&xs[q * win + li]);
            const float xv[4] = {x4.x, x4.y, x4.z, x4.w};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                soap_fma2(acc[q][0], acc[q][1], w[k][0], w[k][1], xv[k], xv[k]);
                soap_fma2(acc[q][2], acc[q][3], w[k][2], w[k][3], xv[k], xv[k]);
            }
        }
    }
}

// conv outputs of the SB spectra and their extrema: per block of 1024 pixels and
// spectrum, the FP32 extrema of A = base - spec (over [0, n)) and C = conv(1 - base) +
// conv(spec) (over [0, n_eff), C != 0) and the magnitudes that bound their rounding
// (blk, order-preserving atomics into mm32).  xs + xi(i) is the staged spectrum value
// of pixel i.  Ends with a block barrier.
template <int SB, bool FULL = false>   // FULL: the tile lies below n_eff (no pixel test needed)
__device__ __forceinline__ void conv32_finish(const float *xs, int win, int xoff, int i0, int ib, int n, int n_eff,
                                              const int *srow, int nsb, const bool (&lv)[FC_PIX],
                                              const float (&acc)[SB][FC_PIX], const float *__restrict__ b32a,
                                              const float *__restrict__ b32b, const float *__restrict__ c32a,
                                              const float *__restrict__ c32b, int b_every, float *__restrict__ conv,
                                              long long conv_stride, unsigned *mm32, float *blk, int nbx, int bx,
                                              unsigned (*red)[4][FC_THREADS / 32]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // the two bases and their convolutions at the thread's pixels, once for all spectra
    float ba[FC_PIX], bb[FC_PIX], ka[FC_PIX], kb[FC_PIX];
    const bool al_b = (((uintptr_t)b32a | (uintptr_t)b32b) & 15) == 0;
    const bool al_c = (((uintptr_t)c32a | (uintptr_t)c32b) & 15) == 0;
    if (al_b && ib + FC_PIX <= n) {
        const float4 u = *reinterpret_cast<const float4 *>(b32a + ib), v = *reinterpret_cast<const float4 *>(b32b + ib);
        ba[0] = u.x, ba[1] = u.y, ba[2] = u.z, ba[3] = u.w;
        bb[0] = v.x, bb[1] = v.y, bb[2] = v.z, bb[3] = v.w;
    } else {
#pragma unroll
        for (int p = 0; p < FC_PIX; ++p) {
            ba[p] = (ib + p < n) ? b32a[ib + p] : 0.f;
            bb[p] = (ib + p < n) ? b32b[ib + p] : 0.f;
        }
    }
    const bool full_e = (ib + FC_PIX <= n_eff);
    if (al_c && full_e) {
        const float4 u = *reinterpret_cast<const float4 *>(c32a + ib), v = *reinterpret_cast<const float4 *>(c32b + ib);
        ka[0] = u.x, ka[1] = u.y, ka[2] = u.z, ka[3] = u.w;
        kb[0] = v.x, kb[1] = v.y, kb[2] = v.z, kb[3] = v.w;
    } else {
#pragma unroll
        for (int p = 0; p < FC_PIX; ++p) {
            ka[p] = (ib + p < n_eff) ? c32a[ib + p] : 0.f;
            kb[p] = (ib + p < n_eff) ? c32b[ib + p] : 0.f;
        }
    }
    const bool vec_out = full_e && (conv_stride % FC_PIX) == 0 && ((uintptr_t)conv & 15) == 0;
#pragma unroll
    for (int q = 0; q < SB; ++q) {
        float mn = INFINITY, mx = -INFINITY, ma = 0.f, mc = 0.f;
        if (q < nsb) {
            const int s = srow[q];
            const bool use_b = (b_every > 0 && (s % b_every) == b_every - 1);
            float *cp = conv + (long long)s * conv_stride;
            float cdv[FC_PIX];
#pragma unroll
            for (int p = 0; p < FC_PIX; ++p) {
                const int i = ib + p;
                if (FULL || i < n) {
                    const float b = use_b ? bb[p] : ba[p], x = xs[q * win + (i - i0) + xoff];
                    mn = fminf(mn, b - x);
                    ma = fmaxf(ma, fabsf(b) + fabsf(x));
                }
                cdv[p] = 0.f;
                if (FULL || i < n_eff) {
                    const float cd = lv[p] ? acc[q][p] : 0.f;
                    cdv[p] = cd;
                    const float cb = use_b ? kb[p] : ka[p];
                    const float c = cb + cd;
                    if (c != 0.f) mx = fmaxf(mx, c);
                    mc = fmaxf(mc, fabsf(cb) + fabsf(cd));
                }
            }
            if (vec_out) {
                *reinterpret_cast<float4 *>(cp + ib) = make_float4(cdv[0], cdv[1], cdv[2], cdv[3]);
            } else {
#pragma unroll
                for (int p = 0; p < FC_PIX; ++p)
                    if (ib + p < n_eff) cp[ib + p] = cdv[p];
            }
        }
        // warp extrema on the order-preserving integer images (exact; the per-thread
        // values hold no NaN, which fminf / fmaxf drop)
        const unsigned rmn = __reduce_min_sync(0xffffffffu, soap_ord32(mn));
        const unsigned rmx = __reduce_max_sync(0xffffffffu, soap_ord32(mx));
        const unsigned rma = __reduce_max_sync(0xffffffffu, soap_ord32(ma));
        const unsigned rmc = __reduce_max_sync(0xffffffffu, soap_ord32(mc));
        if (lane == 0) {
            red[q][0][warp] = rmn;
            red[q][1][warp] = rmx;
            red[q][2][warp] = rma;
            red[q][3][warp] = rmc;
        }
    }
    __syncthreads();
    if (threadIdx.x < nsb) {
        const int q = threadIdx.x, s = srow[q];
        unsigned mn = red[q][0][0], mx = red[q][1][0], ma = red[q][2][0], mc = red[q][3][0];
        for (int w = 1; w < FC_THREADS / 32; ++w) {
            mn = min(mn, red[q][0][w]);
            mx = max(mx, red[q][1][w]);
            ma = max(ma, red[q][2][w]);
            mc = max(mc, red[q][3][w]);
        }
        float *bk = blk + ((long long)s * nbx + bx) * 2;
        bk[0] = soap_dec32(mn);
        bk[1] = soap_dec32(mx);
        if (mn != soap_ord32(INFINITY)) atomicMin(&mm32[4 * s + 0], mn);
        if (mx != soap_ord32(-INFINITY)) atomicMax(&mm32[4 * s + 1], mx);
        atomicMax(&mm32[4 * s + 2], ma);
        atomicMax(&mm32[4 * s + 3], mc);
    }
    __syncthreads();
}

// FAST32 convolution of the spectra, fused with the first min/max pass (plain loads:
// spectra rows that are not 16-byte aligned).  Block = 256 threads x 4 consecutive
// pixels, SB spectra staged in shared memory; every thread walks the taps e in
// [ib - R, ib + 3 + R] (R = the block's reach; the start moved down by up to 3 to a
// 16-byte boundary) four at a time with 16-byte shared loads (conflict-free), one FFMA
// + one ex2 per weight.  Taps beyond a pixel's own reach carry weights below e^-cut of
// its central one; where the thread's taps could leave the reference's window
// [-wid, wid - 2], weights are masked.  Grid (ceil(n / 1024), spectra / SB): blocks
// past n_eff only scan A.
template <int SB>
__global__ void __launch_bounds__(FC_THREADS) k_conv32x(int n, int n_eff, const float *__restrict__ c2a,
                                                        const float *__restrict__ lka, const int *__restrict__ livea,
                                                        const int *__restrict__ rblk, int wid,
                                                        const float *__restrict__ spec, long long spec_stride,
                                                        int n_spec, int halo, const float *__restrict__ b32a,
                                                        const float *__restrict__ b32b, const float *__restrict__ c32a,
                                                        const float *__restrict__ c32b, int b_every,
                                                        float *__restrict__ conv, long long conv_stride,
                                                        unsigned *mm32, float *blk) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *xs = reinterpret_cast<float *>(smem_raw);
    __shared__ unsigned red[SB][4][FC_THREADS / 32];
    const int win = (FC_TILE + 2 * halo + 4 + 3) & ~3;
    const int i0 = blockIdx.x * FC_TILE;
    const int s0 = blockIdx.y * SB;
    const int nsb = min(SB, n_spec - s0);
    for (int q = 0; q < SB; ++q) {
        const float *sp = spec + (long long)(s0 + q) * spec_stride;
        for (int t = threadIdx.x; t < win; t += FC_THREADS) {
            const int m = i0 - halo + t;
            xs[q * win + t] = (q < nsb && m >= 0 && m < n) ? sp[m] : 0.f;
        }
    }
    __syncthreads();
    const int ib = i0 + threadIdx.x * FC_PIX;
    float acc[SB][FC_PIX];
#pragma unroll
    for (int q = 0; q < SB; ++q)
#pragma unroll
        for (int p = 0; p < FC_PIX; ++p) acc[q][p] = 0.f;
    float c2[FC_PIX], lk[FC_PIX];
    bool lv[FC_PIX];
#pragma unroll
    for (int p = 0; p < FC_PIX; ++p) {
        const int i = ib + p;
        lv[p] = (i < n_eff) && livea[i];
        c2[p] = lv[p] ? c2a[i] : 0.f;
        lk[p] = lv[p] ? lka[i] : -200.f;
    }
    const int R = (i0 < n_eff) ? rblk[blockIdx.x] : 0;
    if (R > 0) {
        const int sh = (halo - R) & 3;
        conv32_taps<SB>(xs, win, threadIdx.x * FC_PIX + halo - R - sh, R, sh, wid, c2, lk, acc);
    }
    __shared__ int srow[SB];   // the spectra of the batch
    if (threadIdx.x < SB) srow[threadIdx.x] = s0 + threadIdx.x;
    __syncthreads();
    conv32_finish<SB>(xs, win, halo, i0, ib, n, n_eff, srow, nsb, lv, acc, b32a, b32b, c32a, c32b, b_every, conv,
                      conv_stride, mm32, blk, gridDim.x, blockIdx.x, red);
}

// The same with TMA staging (spectra rows 16-byte aligned, stride a multiple of 4), on a
// persistent grid: block b walks the items b, b + gridDim.x, ... of (spectrum batch,
// pixel tile), batch-major, and copies the next item's rows by cp.async.bulk into the
// other buffer while the current one is convolved.  Staged row r of an item starts at
// source pixel mb = floor4(i0 - halo); pixels outside [0, n) are zeroed by the threads
// once the copy has landed.
template <int SB>
__global__ void __launch_bounds__(FC_THREADS, 3) k_conv32t(int n, int n_eff, const float *__restrict__ c2a,
                                                           const float *__restrict__ lka,
                                                           const int *__restrict__ livea, const int *__restrict__ rblk,
                                                           int wid, const float *__restrict__ spec,
                                                           long long spec_stride, int n_spec, int halo,
                                                           const float *__restrict__ b32a,
                                                           const float *__restrict__ b32b,
                                                           const float *__restrict__ c32a,
                                                           const float *__restrict__ c32b, int b_every,
                                                           float *__restrict__ conv, long long conv_stride,
                                                           unsigned *mm32, float *blk, int nbx, int *status,
                                                           const unsigned char *__restrict__ zero_spec,
                                                           const int *__restrict__ rows, int nrows,
                                                           long long wait_limit, int drop_first) {
    static_assert(SB <= 31, "one bit per spectrum of a batch");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ unsigned red[SB][4][FC_THREADS / 32];
    __shared__ int srow[SB];
    __shared__ unsigned long long bar[2];
    __shared__ int fail;
    const int win = (FC_TILE + 2 * halo + 12 + 3) & ~3;
    float *xbuf = reinterpret_cast<float *>(smem_raw);   // [2][SB][win]
    // the spectra to convolve: rows[0, nrows) (the non-zero ones), or all n_spec; batch
    // bt holds the listed spectra bt * SB ...
    const int nlisted = rows ? nrows : n_spec;
    const int nwalk = (nlisted + SB - 1) / SB;
    const int nitem = nwalk * nbx;   // the host checks that it fits an int
    auto batch_of = [&](int it) { return it / nbx; };
    auto row_id = [&](int bt, int q) { return rows ? rows[bt * SB + q] : bt * SB + q; };
    // staged window of tile x: first source pixel mb (16-byte aligned, <= i0 - halo) and
    // the in-range part [ca, cb) of the staged row, 16-byte aligned at both ends (the
    // row's allocation is padded beyond n to a multiple of 16 bytes)
    auto window = [&](int x, int &mb, int &ca, int &cb) {
        const int wm0 = x * FC_TILE - halo;
        mb = (wm0 >= 0) ? (wm0 & ~3) : -((-wm0 + 3) & ~3);
        ca = max(mb, 0);
        cb = min(mb + win, (n + 3) & ~3);
    };
    // rows of spectra known to be zero (phases without a visible region) are not copied
    // but zeroed in shared memory: their raw rows need not be written
    auto zero_row = [&](int s) { return zero_spec != nullptr && zero_spec[s] != 0; };
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((unsigned)__cvta_generic_to_shared(&bar[0])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((unsigned)__cvta_generic_to_shared(&bar[1])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fail = 0;
    }
    __syncthreads();
    // (warp 0) copy item it's rows into buffer buf: lane q looks up and copies row q, so
    // the lookups' latencies overlap instead of adding up
    auto issue = [&](int it, int buf) {
        const int lane = threadIdx.x & 31;
        const int bt = batch_of(it), x = it % nbx;
        const int nsb = min(SB, nlisted - bt * SB);
        int mb, ca, cb;
        window(x, mb, ca, cb);
        const unsigned bytes = (cb > ca) ? (unsigned)(cb - ca) * 4u : 0u;
        const unsigned bar_a = (unsigned)__cvta_generic_to_shared(&bar[buf]);
        const int sq = (lane < nsb) ? row_id(bt, lane) : 0;
        const bool cp = (lane < nsb) && !zero_row(sq);
        const unsigned ncopy = (unsigned)__popc(__ballot_sync(0xffffffffu, cp));
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (lane == 0)
            asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a),
                         "r"(bytes * ncopy)
                         : "memory");
        __syncwarp();
        // failure-path test: the block's first window is expected but never copied
        if (cp && bytes && !(drop_first && it == (int)blockIdx.x)) {
            const float *src = spec + (long long)sq * spec_stride + ca;
            float *dst = xbuf + ((size_t)buf * SB + lane) * win + (ca - mb);
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    (unsigned)__cvta_generic_to_shared(dst)),
                "l"(src), "r"(bytes), "r"(bar_a)
                : "memory");
        }
    };
    int k = 0, k_fail = -1;
    if (threadIdx.x < 32 && (int)blockIdx.x < nitem) issue(blockIdx.x, 0);
    for (int it = blockIdx.x; it < nitem; it += gridDim.x, ++k) {
        const int bt = batch_of(it), x = it % nbx;
        const int buf = k & 1;
        if (threadIdx.x < 32 && it + (int)gridDim.x < nitem) issue(it + gridDim.x, buf ^ 1);
        const int nsb = min(SB, nlisted - bt * SB);
        // the item's spectra (shared: the epilogue's last step indexes them by thread);
        // written before the barrier below, read after it, rewritten after the epilogue's
        // closing barrier
        if (threadIdx.x < SB) srow[threadIdx.x] = ((int)threadIdx.x < nsb) ? row_id(bt, threadIdx.x) : 0;
        const int i0 = x * FC_TILE;
        int mb, ca, cb;
        window(x, mb, ca, cb);
        const int xo = (i0 - halo) - mb;   // staged index of source pixel i0 - halo, in [0, 3]
        const int ib = i0 + threadIdx.x * FC_PIX;
        float c2[FC_PIX], lk[FC_PIX];
        bool lv[FC_PIX];
#pragma unroll
        for (int p = 0; p < FC_PIX; ++p) {
            const int i = ib + p;
            lv[p] = (i < n_eff) && livea[i];
            c2[p] = lv[p] ? c2a[i] : 0.f;
            lk[p] = lv[p] ? lka[i] : -200.f;
        }
        const int R = (i0 < n_eff) ? rblk[x] : 0;
        const int sh = (halo - R + xo) & 3;
        float *xs = xbuf + (size_t)buf * SB * win;
        bool ok = false;
        const unsigned bar_a = (unsigned)__cvta_generic_to_shared(&bar[buf]);
        for (long long w = 0; w < wait_limit && !ok; ++w) {
            unsigned r;
            asm volatile(
                "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(r)
                : "r"(bar_a), "r"((unsigned)((k >> 1) & 1))
                : "memory");
            ok = (r != 0);
        }
        if (!ok) atomicExch(&fail, 1);
        // rows of zero spectra in this batch (lane q looks up row q)
        const unsigned zmask = __ballot_sync(
            0xffffffffu, (int)(threadIdx.x & 31) < nsb && zero_row(row_id(bt, (int)(threadIdx.x & 31))));
        // zero the staged pixels outside [0, n), and the rows of absent and zero spectra
        if (ca > mb || cb < mb + win || nsb < SB || zmask) {
            for (int q = 0; q < SB; ++q)
                for (int t = threadIdx.x; t < win; t += FC_THREADS) {
                    const int m = mb + t;
                    if (q >= nsb || ((zmask >> q) & 1u) || m < 0 || m >= n) xs[q * win + t] = 0.f;
                }
        }
        __syncthreads();
        if (fail) {
            k_fail = k;
            break;
        }
        float acc[SB][FC_PIX];
#pragma unroll
        for (int q = 0; q < SB; ++q)
#pragma unroll
            for (int p = 0; p < FC_PIX; ++p) acc[q][p] = 0.f;
        // a batch of spectra known to be zero has no taps to sum: its convolution is
        // the base part alone
        const bool zero_batch = (zmask == (1u << nsb) - 1u);
        if (R > 0 && !zero_batch)
            conv32_taps<SB>(xs, win, threadIdx.x * FC_PIX + halo - R - sh + xo, R, sh, wid, c2, lk, acc);
        if (i0 + FC_TILE <= n_eff)   // uniform for the block
            conv32_finish<SB, true>(xs, win, halo + xo, i0, ib, n, n_eff, srow, nsb, lv, acc, b32a, b32b, c32a,
                                    c32b, b_every, conv, conv_stride, mm32, blk, nbx, x, red);
        else
            conv32_finish<SB, false>(xs, win, halo + xo, i0, ib, n, n_eff, srow, nsb, lv, acc, b32a, b32b, c32a,
                                     c32b, b_every, conv, conv_stride, mm32, blk, nbx, x, red);
    }
    if (k_fail >= 0 && threadIdx.x == 0) {
        // a staged copy did not land in time: record it and give the next item's copy,
        // if one was issued, a bounded wait before leaving
        atomicExch(status, 42);
        if ((long long)blockIdx.x + (long long)(k_fail + 1) * gridDim.x < (long long)nitem) {
            const int kb = k_fail + 1;
            const unsigned bar_a = (unsigned)__cvta_generic_to_shared(&bar[kb & 1]);
            for (long long w = 0; w < wait_limit; ++w) {
                unsigned r;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                    "selp.u32 %0, 1, 0, p;\n\t}"
                    : "=r"(r)
                    : "r"(bar_a), "r"((unsigned)((kb >> 1) & 1))
                    : "memory");
                if (r) break;
            }
        }
    }
}

// pass 2 of the fused form: exact FP64 extrema of the candidate pixels of the pixel
// blocks (1024 pixels each) that can hold one.  grid (ceil(nbx / 8), spectra): warp w
// of a block takes pixel block 8 blockIdx.x + w when its FP32 bounds make it a
// candidate (most are not, and their warps leave at once).
__global__ void __launch_bounds__(256) k_refine64x(int n, int n_eff, int nbx, const float *__restrict__ spec,
                                                   long long spec_stride, const double *__restrict__ ba,
                                                   const double *__restrict__ bb, const double *__restrict__ cba,
                                                   const double *__restrict__ cbb, const float *__restrict__ b32a,
                                                   const float *__restrict__ b32b, const float *__restrict__ c32a,
                                                   const float *__restrict__ c32b, int b_every,
                                                   const float *__restrict__ conv, long long conv_stride,
                                                   const unsigned *__restrict__ mm32, const float *__restrict__ blk,
                                                   unsigned long long *mm64, const unsigned char *__restrict__ zero_spec) {
    const int s = blockIdx.y;
    const int x = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (x >= nbx) return;
    if (zero_spec && zero_spec[s]) return;   // extrema of the base alone (k_zero_extrema)
    const float mnA = soap_dec32(mm32[4 * s + 0]), mxC = soap_dec32(mm32[4 * s + 1]);
    const float tolA = ldexpf(soap_dec32(mm32[4 * s + 2]), -21), tolC = ldexpf(soap_dec32(mm32[4 * s + 3]), -21);
    const float *bk = blk + ((long long)s * nbx + x) * 2;
    const bool needA = bk[0] <= mnA + tolA;
    const bool needC = (mm32[4 * s + 1] != 0u) && (bk[1] >= mxC - tolC);
    if (!needA && !needC) return;          // uniform for the warp
    const bool use_b = (b_every > 0 && (s % b_every) == b_every - 1);
    const float *sp = spec + (long long)s * spec_stride;
    const float *bs = use_b ? b32b : b32a;
    const float *cbs = use_b ? c32b : c32a;
    const double *b64 = use_b ? bb : ba;
    const double *c64 = use_b ? cbb : cba;
    const float *cv = conv + (long long)s * conv_stride;
    unsigned long long mn = ~0ULL, mx = 0ULL;
    const int i_end = min(n, (x + 1) * FC_TILE);
    for (int i = x * FC_TILE + lane; i < i_end; i += 32) {
        const float xv = sp[i];
        if (needA && bs[i] - xv <= mnA + tolA) {
            const double a = b64[i] - (double)xv;
            mn = min(mn, soap_ord_enc(a));
        }
        if (needC && i < n_eff) {
            const float cd = cv[i];
            const float c = cbs[i] + cd;
            if (c != 0.f && c >= mxC - tolC) {
                const double cx = c64[i] + (double)cd;
                if (cx != 0.0) mx = max(mx, soap_ord_enc(cx));
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (lane == 0) {
        if (mn != ~0ULL) atomicMin(&mm64[2 * s], mn);
        if (mx != 0ULL) atomicMax(&mm64[2 * s + 1], mx);
    }
}

// Exact FP64 extrema of the spectra whose deficit is zero, one per base: what
// k_refine64x finds for such a spectrum (its candidates hold the extremes of the base
// alone): min over [0, n) of base, max over [0, n_eff) of the base convolution where
// its FP32 and FP64 values are non-zero.  mmz[2 q] / mmz[2 q + 1] for base q, set to
// (~0, sentinel) by k_mm32_init's rule beforehand.  grid (blocks, bases)
__global__ void __launch_bounds__(256) k_zero_extrema(int n, int n_eff, const double *__restrict__ ba,
                                                      const double *__restrict__ bb, const double *__restrict__ cba,
                                                      const double *__restrict__ cbb, const float *__restrict__ c32a,
                                                      const float *__restrict__ c32b, unsigned long long *mmz) {
    const int q = blockIdx.y;
    const double *b64 = q ? bb : ba;
    const double *c64 = q ? cbb : cba;
    const float *c32 = q ? c32b : c32a;
    unsigned long long mn = ~0ULL, mx = 0ULL;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        mn = min(mn, soap_ord_enc(b64[i] - 0.0));
        if (i < n_eff && c32[i] != 0.f) {
            const double cx = c64[i] + 0.0;
            if (cx != 0.0) mx = max(mx, soap_ord_enc(cx));
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (mn != ~0ULL) atomicMin(&mmz[2 * q], mn);
        if (mx != 0ULL) atomicMax(&mmz[2 * q + 1], mx);
    }
}

// The normalised output of a zero spectrum for each of the b_every types (the same for
// every phase: the base alone), as k_factor and k_norm32 form it: out3[t][i], t < 3.
__global__ void k_zero_rows(int n_eff, int b_every, const float *__restrict__ c32a, const float *__restrict__ c32b,
                            const unsigned long long *__restrict__ mmz, double *__restrict__ out3) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = blockIdx.y;
    if (i >= n_eff) return;
    const int q = (b_every > 0 && (t % b_every) == b_every - 1) ? 1 : 0;
    const double mn = soap_ord_dec(mmz[2 * q]), mx = soap_ord_dec(mmz[2 * q + 1]);
    const float f = (float)((1.0 - mn) / mx);
    const float c = (q ? c32b : c32a)[i] + 0.f;
    out3[(size_t)t * n_eff + i] = soap_f32_to_f64(fmaf(-c, f, 1.0f));
}

// extrema of the zero spectra of a chunk from the per-base values
__global__ void k_zero_mm(int n_spec, const unsigned char *__restrict__ zero_spec, int b_every,
                          const unsigned long long *__restrict__ mmz, unsigned long long *mm64) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_spec || !zero_spec[s]) return;
    const int q = (b_every > 0 && (s % b_every) == b_every - 1) ? 1 : 0;
    mm64[2 * s] = mmz[2 * q];
    mm64[2 * s + 1] = mmz[2 * q + 1];
}

// FP64 normalisation constants per spectrum -> FP32 factor
__global__ void k_factor(int n_spec, const unsigned long long *__restrict__ mm64, float *fac, double *minmax_out) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_spec) return;
    double mn = soap_ord_dec(mm64[2 * s]), mx = soap_ord_dec(mm64[2 * s + 1]);
    fac[s] = (float)((1.0 - mn) / mx);
    if (minmax_out) {
        minmax_out[2 * s] = mn;
        minmax_out[2 * s + 1] = mx;
    }
}

// out = 1 - C f on the FP32 pipe, stored as FP64 bits without an FP64 instruction
__global__ void __launch_bounds__(256) k_norm32(int n_eff, const float *__restrict__ c32a,
                                                const float *__restrict__ c32b, int b_every,
                                                const float *__restrict__ conv, long long conv_stride,
                                                const float *__restrict__ fac, double *__restrict__ out,
                                                long long out_stride, const unsigned char *__restrict__ zero_spec,
                                                int skip_zero) {
    int s = blockIdx.y;
    if (skip_zero && zero_spec && zero_spec[s]) return;   // rows the caller has already
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_eff) return;
    bool use_b = (b_every > 0 && (s % b_every) == b_every - 1);
    const float *cbs = use_b ? c32b : c32a;
    const float cd = (zero_spec && zero_spec[s]) ? 0.f : conv[(long long)s * conv_stride + i];
    float c = cbs[i] + cd;
    out[(long long)s * out_stride + i] = soap_f32_to_f64(fmaf(-c, fac[s], 1.0f));
}

// k_norm32 in groups of four pixels: 16-byte loads and stores (n_eff % 4 == 0, strides
// multiples of 4, 16-byte aligned rows); each thread takes NORM_GROUPS groups a block
// apart, their loads issued before their stores
constexpr int NORM_GROUPS = 4;
__global__ void __launch_bounds__(256) k_norm32v(int n_eff, const float *__restrict__ c32a,
                                                 const float *__restrict__ c32b, int b_every,
                                                 const float *__restrict__ conv, long long conv_stride,
                                                 const float *__restrict__ fac, double *__restrict__ out,
                                                 long long out_stride, const unsigned char *__restrict__ zero_spec,
                                                 int skip_zero) {
    const int s = blockIdx.y;
    const bool zs = zero_spec && zero_spec[s];
    if (skip_zero && zs) return;   // rows the caller has already
    const bool use_b = (b_every > 0 && (s % b_every) == b_every - 1);
    const float *cbs = use_b ? c32b : c32a;
    const float *cr = conv + (long long)s * conv_stride;
    const float f = fac[s];
    double *orow = out + (long long)s * out_stride;
    const int i0 = 4 * (blockIdx.x * blockDim.x * NORM_GROUPS + threadIdx.x);
    float4 cb[NORM_GROUPS], cd[NORM_GROUPS];
#pragma unroll
    for (int g = 0; g < NORM_GROUPS; ++g) {
        const int i = i0 + 4 * g * (int)blockDim.x;
        cb[g] = make_float4(0.f, 0.f, 0.f, 0.f);
        cd[g] = cb[g];
        if (i < n_eff) {
            cb[g] = *reinterpret_cast<const float4 *>(cbs + i);
            // a zero spectrum's convolution is zero (not computed, not stored)
            if (!zs) cd[g] = *reinterpret_cast<const float4 *>(cr + i);
        }
    }
#pragma unroll
    for (int g = 0; g < NORM_GROUPS; ++g) {
        const int i = i0 + 4 * g * (int)blockDim.x;
        if (i >= n_eff) continue;
        double2 *o = reinterpret_cast<double2 *>(orow + i);
        o[0] = make_double2(soap_f32_to_f64(fmaf(-(cb[g].x + cd[g].x), f, 1.0f)),
                            soap_f32_to_f64(fmaf(-(cb[g].y + cd[g].y), f, 1.0f)));
        o[1] = make_double2(soap_f32_to_f64(fmaf(-(cb[g].z + cd[g].z), f, 1.0f)),
                            soap_f32_to_f64(fmaf(-(cb[g].w + cd[g].w), f, 1.0f)));
    }
}

namespace soapgb {

static size_t conv_param_bytes(int n_eff) {
    // FAST64: kq, cq (double) + ranges (int2); FAST32: c2, lk, live (4 bytes each) + per-block reach
    return 2 * ((sizeof(double) * (size_t)n_eff + 255) & ~size_t(255)) + ((sizeof(int2) * (size_t)n_eff + 255) & ~size_t(255)) +
           ((sizeof(int) * (size_t)(n_eff / FC_TILE + 2) + 255) & ~size_t(255));
}

size_t resolution_scratch_bytes(int form, int n, int n_eff, int n_spec) {
    size_t b = sizeof(double) * (size_t)n_eff * n_spec + 256;   // conv
    b += sizeof(unsigned long long) * 2 * n_spec + 256;          // min/max
    b += sizeof(unsigned long long) * 4 + 256 + sizeof(int) * ((size_t)n_spec + 2) + 256;   // zero spectra
    if (form != SOAPGB_PLAIN64)
        b += 2 * (sizeof(double) * (size_t)n_eff + 256) + 2 * (conv_param_bytes(n_eff) + 256) +
             2 * sizeof(double) * (size_t)n + 256;   // base convolutions, tap constants, staged bases
    if (form == SOAPGB_FAST32) {
        b += 2 * (sizeof(float) * (size_t)n + 256) + 2 * (sizeof(float) * (size_t)n_eff + 256);   // base32, cb32
        b += sizeof(float) * (size_t)n * n_spec + 256;                                        // FP32 spectra
        b += 16 * (size_t)n_spec + 256 + 4 * (size_t)n_spec + 256;                               // mm32, factor
        b += sizeof(float) * 2 * (size_t)((n + FC_TILE - 1) / FC_TILE) * n_spec + 256;          // block extrema
    }
    (void)n;
    return b;
}

template <typename T, int SB, typename SrcT = double, typename OutT = double>
static int launch_conv_fast(soapgb_ctx *ctx, int n, int n_eff, const double *lam, const SrcT *spec,
                            long long spec_stride, int n_spec, int one_minus, double sigma_v, int wid,
                            double step_mult, double step_exp, double cut, OutT *conv, long long conv_stride,
                            double sig_max, char *param_scratch) {
    // halo: the widest significant reach, at the largest sigma (bounded by the window)
    double cmin = step_exp * step_exp / (2.0 * sig_max * sig_max);
    int r = (int)floor(sqrt(cut / cmin)) + 2;
    int halo = std::min(wid, r);
    if (halo < 1) halo = 1;
    size_t smem = sizeof(T) * (size_t)SB * (FC_TILE + 2 * halo);
    if (smem > 200 * 1024) return set_error(ctx, SOAPGB_ERR_ARG, "convolution window too wide (%d px)", halo);
    if (smem > 48 * 1024)
        SOAP_CUDA(ctx, cudaFuncSetAttribute(k_conv_fast<T, SB, SrcT, OutT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem));
    T *kq = (T *)param_scratch;
    T *cq = (T *)(param_scratch + ((sizeof(T) * (size_t)n_eff + 255) & ~size_t(255)));
    int2 *rng = (int2 *)(param_scratch + 2 * ((sizeof(T) * (size_t)n_eff + 255) & ~size_t(255)));
    const double s1 = soap_sigma_per_lambda(sigma_v);
    const double ka = step_mult / (s1 * sqrt(2. * SOAP_PI)), kb = step_exp * step_exp / (2.0 * s1 * s1);
    const double kr = sqrt(cut / kb);
    SOAP_TRACED(ctx, "conv_params",
                k_conv_params<T><<<grid_for(ctx, n_eff, 256), 256, 0, ctx->stream>>>(n, n_eff, lam, ka, kb, kr, wid,
                                                                                    halo, kq, cq, rng));
    SOAP_LAUNCHED(ctx);
    dim3 g((n_eff + FC_TILE - 1) / FC_TILE, (n_spec + SB - 1) / SB);
    SOAP_TRACED(ctx, "conv64", k_conv_fast<T, SB, SrcT, OutT><<<g, FC_THREADS, smem, ctx->stream>>>(n, n_eff, kq, cq, rng, spec, spec_stride,
                                                                        n_spec, one_minus, halo, conv, conv_stride));
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}

// The base convolution of the FP32 form: FP64 tap constants (k_conv_params), then
// k_conv_base_df.  Same constants and ranges as launch_conv_fast<double>.
template <int SB>
static int launch_conv_base_df(soapgb_ctx *ctx, int n, int n_eff, const double *lam, const double *spec,
                               long long spec_stride, int n_spec, double sigma_v, int wid, double step_mult,
                               double step_exp, double cut, double *conv, long long conv_stride, double sig_max,
                               char *param_scratch) {
    const double cmin = step_exp * step_exp / (2.0 * sig_max * sig_max);
    const int r = (int)floor(sqrt(cut / cmin)) + 2;
    int halo = std::min(wid, r);
    if (halo < 1) halo = 1;
    const size_t smem = sizeof(float2) * (size_t)SB * (FC_TILE + 2 * halo);
    if (smem > 200 * 1024) return set_error(ctx, SOAPGB_ERR_ARG, "convolution window too wide (%d px)", halo);
    if (smem > 48 * 1024)
        SOAP_CUDA(ctx, cudaFuncSetAttribute(k_conv_base_df<SB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    double *kq = (double *)param_scratch;
    double *cq = (double *)(param_scratch + ((sizeof(double) * (size_t)n_eff + 255) & ~size_t(255)));
    int2 *rng = (int2 *)(param_scratch + 2 * ((sizeof(double) * (size_t)n_eff + 255) & ~size_t(255)));
    const double s1 = soap_sigma_per_lambda(sigma_v);
    const double ka = step_mult / (s1 * sqrt(2. * SOAP_PI)), kb = step_exp * step_exp / (2.0 * s1 * s1);
    const double kr = sqrt(cut / kb);
    SOAP_TRACED(ctx, "conv_params",
                k_conv_params<double><<<grid_for(ctx, n_eff, 256), 256, 0, ctx->stream>>>(n, n_eff, lam, ka, kb, kr,
                                                                                         wid, halo, kq, cq, rng));
    SOAP_LAUNCHED(ctx);
    const dim3 g((n_eff + FC_TILE - 1) / FC_TILE, (n_spec + SB - 1) / SB);
    SOAP_TRACED(ctx, "conv_base", k_conv_base_df<SB><<<g, FC_THREADS, smem, ctx->stream>>>(
                                      n, n_eff, kq, cq, rng, spec, spec_stride, n_spec, halo, conv, conv_stride));
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}

// FP32 tap constants (from the FP64 ones of the base convolution when given) and the
// reach of every block of 1024 pixels; returns the staging halo
static int conv32_params(soapgb_ctx *ctx, int n, int n_eff, const double *lam, double sigma_v, int wid,
                         double step_mult, double step_exp, double cut, double sig_max, char *param_scratch,
                         const char *params64, int *halo_out) {
    double cmin = step_exp * step_exp / (2.0 * sig_max * sig_max);
    int r = (int)floor(sqrt(cut / cmin)) + 2;
    int halo = std::min(wid, r);
    if (halo < 1) halo = 1;
    *halo_out = halo;
    const size_t pb = (sizeof(float) * (size_t)n_eff + 255) & ~size_t(255);
    float *c2 = (float *)param_scratch;
    float *lk = (float *)(param_scratch + pb);
    int *live = (int *)(param_scratch + 2 * pb);
    int *rblk = (int *)(param_scratch + 3 * pb);
    const int nbx = (n + FC_TILE - 1) / FC_TILE;
    SOAP_CUDA(ctx, cudaMemsetAsync(rblk, 0, sizeof(int) * (size_t)nbx, ctx->stream));
    if (params64) {   // from the FP64 constants of the base convolution (kq, cq, ranges)
        const size_t pb64 = (sizeof(double) * (size_t)n_eff + 255) & ~size_t(255);
        SOAP_TRACED(ctx, "conv_params",
                    k_conv32_derive<<<grid_for(ctx, n_eff, 256), 256, 0, ctx->stream>>>(
                        n_eff, (const double *)params64, (const double *)(params64 + pb64),
                        (const int2 *)(params64 + 2 * pb64), halo, (float)cut, c2, lk, live, rblk));
    } else {
        SOAP_TRACED(ctx, "conv_params",
                    k_conv32_params<<<grid_for(ctx, n_eff, 256), 256, 0, ctx->stream>>>(
                        n, n_eff, lam, sigma_v, wid, halo, step_mult, step_exp, cut, c2, lk, live, rblk));
    }
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}

// FAST32 convolution of n_spec spectra fused with the first extrema pass (k_conv32t
// with TMA staging for 16-byte aligned rows, else k_conv32x); tap constants from
// conv32_params
static int conv32_run(soapgb_ctx *ctx, int n, int n_eff, int wid, int halo, const char *param_scratch,
                      const float *spec, long long spec_stride, int n_spec, const float *b32a, const float *b32b,
                      const float *c32a, const float *c32b, int b_every, float *conv, unsigned *mm32, float *blk,
                      const unsigned char *zero_spec, const int *rows, int nrows) {
    constexpr int SB = 8;
    const size_t pb = (sizeof(float) * (size_t)n_eff + 255) & ~size_t(255);
    const float *c2 = (const float *)param_scratch;
    const float *lk = (const float *)(param_scratch + pb);
    const int *live = (const int *)(param_scratch + 2 * pb);
    const int *rblk = (const int *)(param_scratch + 3 * pb);
    const int nbx = (n + FC_TILE - 1) / FC_TILE;
    const int nbatch = (n_spec + SB - 1) / SB;
    if (spec_stride % 4 == 0 && ((uintptr_t)spec & 15) == 0) {
        // TMA staging, double buffered: a block keeps its tile over several spectrum batches
        const int win_t = (FC_TILE + 2 * halo + 12 + 3) & ~3;
        size_t smem_t = sizeof(float) * 2 * (size_t)SB * win_t;
        if (smem_t > 200 * 1024) return set_error(ctx, SOAPGB_ERR_ARG, "convolution window too wide (%d px)", halo);
        SOAP_CUDA(ctx, cudaFuncSetAttribute(k_conv32t<SB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_t));
        const int nwalk = rows ? (nrows + SB - 1) / SB : nbatch;
        if (nwalk == 0) return SOAPGB_OK;   // every spectrum is zero
        int per_sm = 0;
        SOAP_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conv32t<SB>, FC_THREADS, smem_t));
        const long long nitem = (long long)nwalk * nbx;
        if (nitem > 0x7fffffffLL) return set_error(ctx, SOAPGB_ERR_ARG, "convolution: too many (batch, tile) items");
        const int g = (int)std::max<long long>(1, std::min<long long>(nitem, (long long)std::max(per_sm, 1) *
                                                                                  std::max(ctx->num_sms, 1)));
        SOAP_TRACED(ctx, "conv32", k_conv32t<SB><<<g, FC_THREADS, smem_t, ctx->stream>>>(n, n_eff, c2, lk, live, rblk, wid, spec, spec_stride,
                                                              n_spec, halo, b32a, b32b, c32a, c32b, b_every, conv,
                                                              n_eff, mm32, blk, nbx, ctx->d_status, zero_spec,
                                                              rows, nrows,
                                                              ctx->test_wait_limit > 0 ? ctx->test_wait_limit
                                                                                       : (1LL << 24),
                                                              ctx->test_drop_copy == 2 ? 1 : 0));
    } else {
        const int win = (FC_TILE + 2 * halo + 4 + 3) & ~3;
        size_t smem = sizeof(float) * (size_t)SB * win;
        if (smem > 200 * 1024) return set_error(ctx, SOAPGB_ERR_ARG, "convolution window too wide (%d px)", halo);
        if (smem > 48 * 1024)
            SOAP_CUDA(ctx, cudaFuncSetAttribute(k_conv32x<SB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        dim3 g(nbx, nbatch);
        SOAP_TRACED(ctx, "conv32", k_conv32x<SB><<<g, FC_THREADS, smem, ctx->stream>>>(n, n_eff, c2, lk, live, rblk, wid, spec, spec_stride,
                                                           n_spec, halo, b32a, b32b, c32a, c32b, b_every, conv, n_eff,
                                                           mm32, blk));
    }
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}

__global__ void k_f64_to_f32(long long count, const double *__restrict__ a, float *out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) out[i] = (float)a[i];
}

static char *carve(char *&p, size_t bytes) {
    char *r = p;
    p += (bytes + 255) & ~size_t(255);
    return r;
}

int resolution32_prepare(soapgb_ctx *ctx, int n, int n_eff, int n_spec, const double *d_wave, double wave0,
                         double wave1, double wave_last, const double *base_a, const double *base_b, int b_every,
                         double sigma_v, double window, double step_mult, double step_exp, double sentinel,
                         char *scratch, Res32 &R) {
    if (!base_a) return set_error(ctx, SOAPGB_ERR_ARG, "FP32 resolution needs a base spectrum");
    const int wid = conv_halfwidth(wave0, wave1, sigma_v, window);
    char *p = scratch;
    R.n = n;
    R.n_eff = n_eff;
    R.n_spec = n_spec;
    R.wid = wid;
    R.b_every = b_every;
    R.sentinel = sentinel;
    R.base_a = base_a;
    R.base_b = (base_b && b_every > 0) ? base_b : nullptr;
    R.conv32 = (float *)carve(p, sizeof(double) * (size_t)n_eff * n_spec);
    R.mm = (unsigned long long *)carve(p, sizeof(unsigned long long) * 2 * n_spec);
    // the largest sigma (sigma grows with wavelength) sets the widest reach
    const double lmax = std::max(std::fabs(wave0), std::fabs(wave_last)) * 1.001;
    const double sig_max = -1 * lmax * (1 - sqrt((1 + sigma_v / SOAP_C_LIGHT) / (1 - sigma_v / SOAP_C_LIGHT)));
    if (!(sig_max > 0)) return set_error(ctx, SOAPGB_ERR_ARG, "non-positive instrument sigma");
    char *pscr = carve(p, conv_param_bytes(n_eff));     // FP64 tap constants of the base convolution
    char *pscr32 = carve(p, conv_param_bytes(n_eff));   // FP32 tap constants of the spectra's
    int rc;
    double *cb_a, *cb_b = nullptr;
    if (R.base_b) {
        // both bases in one launch (the FP64 weights are shared): staged as rows of one array
        double *bb = (double *)carve(p, sizeof(double) * 2 * (size_t)n);
        double *cb = (double *)carve(p, sizeof(double) * 2 * (size_t)n_eff);
        SOAP_CUDA(ctx, cudaMemcpyAsync(bb, base_a, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(bb + n, base_b, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
        rc = launch_conv_base_df<2>(ctx, n, n_eff, d_wave, bb, n, 2, sigma_v, wid, step_mult, step_exp, 40.0, cb,
                                    n_eff, sig_max, pscr);
        if (rc) return rc;
        cb_a = cb;
        cb_b = cb + n_eff;
    } else {
        cb_a = (double *)carve(p, sizeof(double) * (size_t)n_eff);
        rc = launch_conv_base_df<1>(ctx, n, n_eff, d_wave, base_a, 0, 1, sigma_v, wid, step_mult, step_exp, 40.0,
                                    cb_a, 0, sig_max, pscr);
        if (rc) return rc;
    }
    R.cb_a = cb_a;
    R.cb_b = cb_b;
    float *b32a = (float *)carve(p, sizeof(float) * (size_t)n);
    float *b32b = (float *)carve(p, sizeof(float) * (size_t)n);
    float *c32a = (float *)carve(p, sizeof(float) * (size_t)n_eff);
    float *c32b = (float *)carve(p, sizeof(float) * (size_t)n_eff);
    R.mm32 = (unsigned *)carve(p, 16 * (size_t)n_spec);
    R.fac = (float *)carve(p, 4 * (size_t)n_spec);
    R.nbx = (n + FC_TILE - 1) / FC_TILE;   // extrema blocks of 1024 pixels
    R.blk = (float *)carve(p, sizeof(float) * 2 * (size_t)R.nbx * n_spec);
    k_base_prep<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, n_eff, base_a, cb_a, b32a, c32a);
    SOAP_LAUNCHED(ctx);
    if (cb_b) {
        k_base_prep<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, n_eff, base_b, cb_b, b32b, c32b);
        SOAP_LAUNCHED(ctx);
    }
    R.b32a = b32a;
    R.b32b = cb_b ? b32b : b32a;
    R.c32a = c32a;
    R.c32b = cb_b ? c32b : c32a;
    rc = conv32_params(ctx, n, n_eff, d_wave, sigma_v, wid, step_mult, step_exp, 30.0, sig_max, pscr32, pscr,
                       &R.halo);
    if (rc) return rc;
    R.p32 = pscr32;
    // extrema of the zero spectra, per base
    R.mmz = (unsigned long long *)carve(p, sizeof(unsigned long long) * 4);
    R.blist = (int *)carve(p, sizeof(int) * ((size_t)n_spec + 2));
    k_mm32_init<<<1, 32, 0, ctx->stream>>>(2, sentinel, nullptr, R.mmz);
    SOAP_LAUNCHED(ctx);
    k_zero_extrema<<<dim3(std::max(1, std::min(grid_for(ctx, n, 256), 4 * std::max(ctx->num_sms, 1))), R.base_b ? 2 : 1),
                     256, 0, ctx->stream>>>(n, n_eff, base_a, R.base_b ? R.base_b : base_a, cb_a, cb_b ? cb_b : cb_a,
                                            c32a, cb_b ? c32b : c32a, R.mmz);
    SOAP_LAUNCHED(ctx);
    R.next = p;
    return SOAPGB_OK;
}

int resolution32_run(soapgb_ctx *ctx, const Res32 &R, const float *spec32, long long spec_stride, int s0, int s1,
                     double *d_out, long long out_stride, double *d_minmax, const unsigned char *zero_spec,
                     const unsigned char *zero_host, ZeroRows zero_rows, const int *blist_pre, int nlist_pre) {
    const int ns = s1 - s0;
    if (ns <= 0) return SOAPGB_OK;
    if (R.b_every > 0 && s0 % R.b_every != 0)
        return set_error(ctx, SOAPGB_ERR_ARG, "resolution chunk must start at a multiple of %d spectra", R.b_every);
    const int n = R.n, n_eff = R.n_eff;
    const float *sp = spec32 + (long long)s0 * spec_stride;
    float *conv = R.conv32 + (long long)s0 * n_eff;
    unsigned *mm32 = R.mm32 + 4LL * s0;
    unsigned long long *mm = R.mm + 2LL * s0;
    float *fac = R.fac + s0;
    float *blk = R.blk + 2LL * R.nbx * s0;
    k_mm32_init<<<(ns + 127) / 128, 128, 0, ctx->stream>>>(ns, R.sentinel, mm32, mm);
    SOAP_LAUNCHED(ctx);
    // spectra known to be zero (both flag copies given): their batches are left out of
    // the convolution and their extrema come from the bases
    const unsigned char *zs = (zero_spec && zero_host) ? zero_spec + s0 : nullptr;
    // the non-zero spectra of the chunk (relative indices): only they are convolved, in
    // batches of 8 without zero rows
    const int *blist = nullptr;
    int nlist = 0;
    if (zs && blist_pre) {   // the caller uploaded the list with its own small inputs
        blist = blist_pre;
        nlist = nlist_pre;
        k_zero_mm<<<(ns + 127) / 128, 128, 0, ctx->stream>>>(ns, zs, R.b_every, R.mmz, mm);
        SOAP_LAUNCHED(ctx);
    } else if (zs) {
        std::vector<int> bl;
        for (int q = 0; q < ns; ++q)
            if (!zero_host[s0 + q]) bl.push_back(q);
        nlist = (int)bl.size();
        if (nlist > 0)   // pageable source: staged by the driver before the call returns
            SOAP_CUDA(ctx, cudaMemcpyAsync(R.blist, bl.data(), sizeof(int) * nlist, cudaMemcpyHostToDevice, ctx->stream));
        blist = R.blist;
        k_zero_mm<<<(ns + 127) / 128, 128, 0, ctx->stream>>>(ns, zs, R.b_every, R.mmz, mm);
        SOAP_LAUNCHED(ctx);
    }
    int rc = conv32_run(ctx, n, n_eff, R.wid, R.halo, R.p32, sp, spec_stride, ns, R.b32a, R.b32b, R.c32a, R.c32b,
                        R.b_every, conv, mm32, blk, zs, blist, nlist);
    if (rc) return rc;
    // the zero spectra's rows are left unwritten where the caller has them already
    const bool skip_zero = zs && zero_rows == ZeroRows::SKIP;
    double *out = d_out + (long long)s0 * out_stride;
    SOAP_TRACED(ctx, "refine64",
                k_refine64x<<<dim3((R.nbx + 7) / 8, ns), 256, 0, ctx->stream>>>(n, n_eff, R.nbx, sp, spec_stride, R.base_a, R.base_b,
                                                         R.cb_a, R.cb_b, R.b32a, R.b32b, R.c32a, R.c32b, R.b_every,
                                                         conv, n_eff, mm32, blk, mm, zs));
    SOAP_LAUNCHED(ctx);
    k_factor<<<(ns + 127) / 128, 128, 0, ctx->stream>>>(ns, mm, fac, d_minmax ? d_minmax + 2LL * s0 : nullptr);
    SOAP_LAUNCHED(ctx);
    if (n_eff % 4 == 0 && out_stride % 2 == 0 && ((uintptr_t)out & 15) == 0) {
        dim3 g3((unsigned)((n_eff / 4 + 256 * NORM_GROUPS - 1) / (256 * NORM_GROUPS)), ns);
        SOAP_TRACED(ctx, "norm32", k_norm32v<<<g3, 256, 0, ctx->stream>>>(n_eff, R.c32a, R.c32b, R.b_every, conv,
                                                                           n_eff, fac, out, out_stride, zs,
                                                                           skip_zero ? 1 : 0));
    } else {
        dim3 g3(grid_for(ctx, n_eff, 256), ns);
        SOAP_TRACED(ctx, "norm32", k_norm32<<<g3, 256, 0, ctx->stream>>>(n_eff, R.c32a, R.c32b, R.b_every, conv,
                                                                          n_eff, fac, out, out_stride, zs,
                                                                          skip_zero ? 1 : 0));
    }
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}

int resolution32_zero_rows(soapgb_ctx *ctx, const Res32 &R, int n_types, double *out) {
    k_zero_rows<<<dim3(grid_for(ctx, R.n_eff, 256), n_types), 256, 0, ctx->stream>>>(R.n_eff, R.b_every, R.c32a,
                                                                                       R.c32b, R.mmz, out);
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}

int resolution_device(soapgb_ctx *ctx, int form, int n, int n_eff, int n_spec, const double *d_wave, double wave0,
                      double wave1, double wave_last, const void *d_spec_v, int spec_f32, long long spec_stride,
                      const double *base_a, const double *base_b, int b_every, double sigma_v, double window,
                      double step_mult, double step_exp, double sentinel, double *d_out, long long out_stride,
                      double *d_minmax, char *scratch) {
    if (form == SOAPGB_FAST32 && base_a) {
        // ---- FP32 pipe throughout, exact FP64 normalisation constants ----------------
        Res32 R;
        int rc = resolution32_prepare(ctx, n, n_eff, n_spec, d_wave, wave0, wave1, wave_last, base_a, base_b,
                                      b_every, sigma_v, window, step_mult, step_exp, sentinel, scratch, R);
        if (rc) return rc;
        const float *spec32 = (const float *)d_spec_v;
        if (!spec_f32) {
            char *p = R.next;
            float *tmp = (float *)carve(p, sizeof(float) * (size_t)n * n_spec);
            const double *ds = (const double *)d_spec_v;
            for (int q = 0; q < n_spec; ++q) {
                k_f64_to_f32<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, ds + (long long)q * spec_stride,
                                                                            tmp + (long long)q * n);
                SOAP_LAUNCHED(ctx);
            }
            spec32 = tmp;
            spec_stride = n;
        }
        return resolution32_run(ctx, R, spec32, spec_stride, 0, n_spec, d_out, out_stride, d_minmax);
    }
    int wid = conv_halfwidth(wave0, wave1, sigma_v, window);
    char *p = scratch;
    double *conv = (double *)carve(p, sizeof(double) * (size_t)n_eff * n_spec);
    unsigned long long *mm = (unsigned long long *)carve(p, sizeof(unsigned long long) * 2 * n_spec);
    double *cb_a = nullptr, *cb_b = nullptr;
    const double *d_spec = (const double *)d_spec_v;
    if (spec_f32 && form != SOAPGB_FAST32)
        return set_error(ctx, SOAPGB_ERR_ARG, "FP32 spectra are accepted by the FP32 form only");
    if (form == SOAPGB_PLAIN64) {
        dim3 g(grid_for(ctx, n_eff, 256), n_spec);
        SOAP_TRACED(ctx, "conv_plain64", k_conv_plain64<<<g, 256, 0, ctx->stream>>>(n, n_eff, d_wave, d_spec, spec_stride, base_a, base_b, b_every,
                                                   sigma_v, wid, step_mult, step_exp, conv, n_eff));
        SOAP_LAUNCHED(ctx);
    } else {
        // the largest sigma (sigma grows with wavelength) sets the widest reach
        double lmax = std::max(std::fabs(wave0), std::fabs(wave_last)) * 1.001;
        double sig_max = -1 * lmax * (1 - sqrt((1 + sigma_v / SOAP_C_LIGHT) / (1 - sigma_v / SOAP_C_LIGHT)));
        if (!(sig_max > 0)) return set_error(ctx, SOAPGB_ERR_ARG, "non-positive instrument sigma");
        double cut = (form == SOAPGB_FAST32) ? 30.0 : 40.0;
        int rc;
        char *pscr = carve(p, conv_param_bytes(n_eff));     // FP64 tap constants of the base convolution
        char *pscr32 = carve(p, conv_param_bytes(n_eff));   // FP32 tap constants of the spectra's
        if (base_a && base_b && b_every > 0) {
            // both bases in one launch (the FP64 weights are shared): staged as rows of one array
            double *bb = (double *)carve(p, sizeof(double) * 2 * (size_t)n);
            double *cb = (double *)carve(p, sizeof(double) * 2 * (size_t)n_eff);
            SOAP_CUDA(ctx, cudaMemcpyAsync(bb, base_a, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
            SOAP_CUDA(ctx, cudaMemcpyAsync(bb + n, base_b, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
            rc = launch_conv_fast<double, 2>(ctx, n, n_eff, d_wave, bb, n, 2, 1, sigma_v, wid, step_mult, step_exp,
                                             40.0, cb, n_eff, sig_max, pscr);
            if (rc) return rc;
            cb_a = cb;
            cb_b = cb + n_eff;
        } else if (base_a) {
            cb_a = (double *)carve(p, sizeof(double) * (size_t)n_eff);
            rc = launch_conv_fast<double, 1>(ctx, n, n_eff, d_wave, base_a, 0, 1, 1, sigma_v, wid, step_mult,
                                             step_exp, 40.0, cb_a, 0, sig_max, pscr);
            if (rc) return rc;
        }
        // FAST64, or no base (the whole (1 - A) is convolved): FP64
        rc = launch_conv_fast<double, 4>(ctx, n, n_eff, d_wave, d_spec, spec_stride, n_spec, base_a ? 0 : 1,
                                         sigma_v, wid, step_mult, step_exp, base_a ? cut : 40.0, conv, n_eff,
                                         sig_max, pscr);
        if (rc) return rc;
    }
    k_minmax_init<<<(n_spec + 127) / 128, 128, 0, ctx->stream>>>(n_spec, sentinel, mm);
    SOAP_LAUNCHED(ctx);
    {
        int bx = std::max(1, std::min(64, (n + 255) / 256));
        dim3 g(bx, n_spec);
        SOAP_TRACED(ctx, "minmax64", k_minmax<<<g, 256, 0, ctx->stream>>>(n, n_eff, d_spec, spec_stride, base_a, base_b, b_every, conv, n_eff,
                                             cb_a, cb_b, mm));
        SOAP_LAUNCHED(ctx);
    }
    {
        dim3 g(grid_for(ctx, n_eff, 256), n_spec);
        SOAP_TRACED(ctx, "norm64", k_norm<<<g, 256, 0, ctx->stream>>>(n_eff, conv, n_eff, mm, d_out, out_stride, d_minmax,
                                           form == SOAPGB_PLAIN64));
        SOAP_LAUNCHED(ctx);
    }
    return SOAPGB_OK;
}

}  // namespace soapgb

extern "C" int soapgb_lower_resolution(soapgb_ctx *ctx, int form, int n, int n_eff, int n_spec, const double *wave,
                                       const double *base, const double *spec, double sigma_v, double window,
                                       double step_mult, double step_exp, double sentinel, int mem, double *out,
                                       double *minmax_out) {
    if (!ctx) return SOAPGB_ERR_ARG;
    if (n < 3 || n_eff < 1 || n_eff > n || n_spec < 0 || !wave || !spec || !out || !(sigma_v > 0) ||
        !(step_exp > 0))
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_lower_resolution: bad arguments");
    if (form != SOAPGB_PLAIN64 && form != SOAPGB_FAST64 && form != SOAPGB_FAST32)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_lower_resolution: unknown form %d", form);
    if (n_spec == 0) return SOAPGB_OK;
    SOAP_DEVICE(ctx);
    bool host = (mem == SOAPGB_HOST);
    double w01[3];
    if (host) {
        w01[0] = wave[0];
        w01[1] = wave[1];
        w01[2] = wave[n_eff - 1];
    } else {
        SOAP_CUDA(ctx, cudaMemcpyAsync(w01, wave, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(w01 + 2, wave + n_eff - 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    int wid = conv_halfwidth(w01[0], w01[1], sigma_v, window);
    if (wid < 1 || 2 * wid + 2 >= n)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_lower_resolution: convolution half width %d invalid for n=%d", wid, n);
    Workspace ws(ctx);
    int s_wave = ws.add(host ? sizeof(double) * n : 0);
    int s_base = ws.add(host && base ? sizeof(double) * n : 0);
    int s_spec = ws.add(host ? sizeof(double) * (size_t)n * n_spec : 0);
    int s_out = ws.add(host ? sizeof(double) * (size_t)n_eff * n_spec : 0);
    int s_mm = ws.add(host && minmax_out ? sizeof(double) * 2 * n_spec : 0);
    int s_scr = ws.add(resolution_scratch_bytes(form, n, n_eff, n_spec));
    int rc = ws.commit();
    if (rc) return rc;
    const double *d_wave = (const double *)stage_in(ctx, mem, wave, sizeof(double) * n, ws.get<void>(s_wave), &rc);
    if (rc) return rc;
    const double *d_base = (const double *)stage_in(ctx, mem, base, base ? sizeof(double) * n : 0, ws.get<void>(s_base), &rc);
    if (rc) return rc;
    const double *d_spec = (const double *)stage_in(ctx, mem, spec, sizeof(double) * (size_t)n * n_spec, ws.get<void>(s_spec), &rc);
    if (rc) return rc;
    double *d_out = host ? ws.get<double>(s_out) : out;
    double *d_mm = minmax_out ? (host ? ws.get<double>(s_mm) : minmax_out) : nullptr;
    rc = resolution_device(ctx, form, n, n_eff, n_spec, d_wave, w01[0], w01[1], w01[2], d_spec, 0, n, d_base, nullptr, 0,
                           sigma_v, window, step_mult, step_exp, sentinel, d_out, n_eff, d_mm, ws.get<char>(s_scr));
    if (rc) return rc;
    if (host) {
        SOAP_CUDA(ctx, cudaMemcpyAsync(out, d_out, sizeof(double) * (size_t)n_eff * n_spec, cudaMemcpyDeviceToHost, ctx->stream));
        if (minmax_out)
            SOAP_CUDA(ctx, cudaMemcpyAsync(minmax_out, d_mm, sizeof(double) * 2 * n_spec, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return host ? check_status(ctx, "soapgb_lower_resolution") : SOAPGB_OK;
}

// ---------------------------------------------------------------------------
// Adjoint of the PLAIN64 resolution step (the differentiable form; the reference
// has no gradient path).  Per spectrum, with f = (1 - mn) / mx and S = sum_i G_i C_i
// (G the gradient of a scalar w.r.t. out):
//   dL/dC_i = -f G_i + [i = i_max] S (1 - mn) / mx^2
//   dL/dA_m = -sum_i K(i, m) dL/dC_i + [m = i_min] S / mx
// with K(i, m) = step_mult e^{-(m-i)^2 step_exp^2 / (2 s_i^2)} / (s_i sqrt(2 pi)) on the
// interior pixels i (m - i in [-w, w-2]), and i_min / i_max the first pixels holding
// min A and max C (the subgradient at ties; a maximum that stayed at the sentinel has
// no pixel and no gradient).  dL/dspec = -dL/dA with a base, dL/dA without;
// dL/dbase = sum over the spectra of dL/dA, in spectrum order.
// ---------------------------------------------------------------------------
// tap constants per pixel: kq = step_mult / (s_i sqrt(2 pi)), cq = step_exp^2 / (2 s_i^2)
// on the interior pixels, kq = 0 elsewhere
__global__ void k_radj_taps(int n, int n_eff, const double *__restrict__ lam, double sigma_v, int wid,
                            double step_mult, double step_exp, double *__restrict__ kq, double *__restrict__ cq) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_eff) return;
    double k = 0.0, c = 0.0;
    if (i > wid && i + wid < n - 1) {
        const double sig = soap_delta_lambda(sigma_v, lam[i]);
        k = step_mult / (sig * sqrt(2.0 * SOAP_PI));
        c = step_exp * step_exp / (2.0 * sig * sig);
    }
    kq[i] = k;
    cq[i] = c;
}

constexpr int RADJ_THREADS = 512;

// one block per spectrum: S in a fixed tree order, the first extremum pixels by min
__global__ void __launch_bounds__(RADJ_THREADS) k_radj_reduce(int n, int n_eff, const double *__restrict__ spec,
                                                               const double *__restrict__ base,
                                                               const double *__restrict__ conv,
                                                               const unsigned long long *__restrict__ mm,
                                                               const double *__restrict__ g, double *par, int *idx) {
    const int s = blockIdx.x, t = threadIdx.x;
    const double *sp = spec + (long long)s * n;
    const double *cp = conv + (long long)s * n_eff;
    const double *gp = g + (long long)s * n_eff;
    const double mn = soap_ord_dec(mm[2 * s]), mx = soap_ord_dec(mm[2 * s + 1]);
    double acc = 0.0;
    int im = INT_MAX, ix = INT_MAX;
    for (int i = t; i < n; i += RADJ_THREADS) {
        const double a = base ? __dsub_rn(base[i], sp[i]) : sp[i];
        if (a == mn && im == INT_MAX) im = i;
        if (i < n_eff) {
            const double c = cp[i];
            acc = fma(gp[i], c, acc);
            if (c != 0.0 && c == mx && ix == INT_MAX) ix = i;
        }
    }
    __shared__ double sh[RADJ_THREADS];
    __shared__ int si[RADJ_THREADS], sx[RADJ_THREADS];
    sh[t] = acc;
    si[t] = im;
    sx[t] = ix;
    __syncthreads();
    for (int o = RADJ_THREADS / 2; o > 0; o >>= 1) {
        if (t < o) {
            sh[t] += sh[t + o];
            si[t] = min(si[t], si[t + o]);
            sx[t] = min(sx[t], sx[t + o]);
        }
        __syncthreads();
    }
    if (t == 0) {
        const double S = sh[0];
        par[3 * s] = (1.0 - mn) / mx;
        par[3 * s + 1] = S / mx;
        par[3 * s + 2] = S * (1.0 - mn) / (mx * mx);
        idx[2 * s] = si[0] == INT_MAX ? -1 : si[0];
        idx[2 * s + 1] = sx[0] == INT_MAX ? -1 : sx[0];
    }
}

// the transposed tap gather, one thread per (pixel m, spectrum)
__global__ void __launch_bounds__(256) k_radj_spec(int n, int n_eff, int wid, const double *__restrict__ kq,
                                                   const double *__restrict__ cq, const double *__restrict__ g,
                                                   const double *__restrict__ par, const int *__restrict__ idx,
                                                   int has_base, double *__restrict__ grad_spec) {
    const int s = blockIdx.y;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const double f = par[3 * s], dmn = par[3 * s + 1], dmx = par[3 * s + 2];
    const int imin = idx[2 * s], imax = idx[2 * s + 1];
    const double *gp = g + (long long)s * n_eff;
    const int lo = max(m - wid + 2, 0), hi = min(m + wid, n_eff - 1);
    double acc = 0.0;
    for (int i = lo; i <= hi; ++i) {
        const double k = kq[i];
        if (k == 0.0) continue;
        const double d = (double)(m - i);
        double gc = -f * gp[i];
        if (i == imax) gc += dmx;
        acc = fma(k * exp(-d * d * cq[i]), gc, acc);
    }
    const double ga = (m == imin ? dmn : 0.0) - acc;
    grad_spec[(long long)s * n + m] = has_base ? -ga : ga;
}

// dL/dbase[m] = sum_s dL/dA_s[m] = -sum_s grad_spec[s][m] (with a base), spectra in order
__global__ void k_radj_base(int n, int n_spec, const double *__restrict__ grad_spec, double *__restrict__ grad_base) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    double acc = 0.0;
    for (int s = 0; s < n_spec; ++s) acc -= grad_spec[(long long)s * n + m];
    grad_base[m] = acc;
}

extern "C" int soapgb_lower_resolution_adjoint(soapgb_ctx *ctx, int n, int n_eff, int n_spec, const double *wave,
                                               const double *base, const double *spec, double sigma_v,
                                               double window, double step_mult, double step_exp, double sentinel,
                                               const double *g_out, int mem, double *grad_spec,
                                               double *grad_base) {
    if (!ctx) return SOAPGB_ERR_ARG;
    if (n < 3 || n_eff < 1 || n_eff > n || n_spec < 0 || !wave || !spec || !g_out || !grad_spec ||
        !(sigma_v > 0) || !(step_exp > 0) || (grad_base && !base))
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_lower_resolution_adjoint: bad arguments");
    SOAP_DEVICE(ctx);
    const bool host = (mem == SOAPGB_HOST);
    if (n_spec == 0) {
        if (grad_base) {
            if (host) std::fill(grad_base, grad_base + n, 0.0);
            else SOAP_CUDA(ctx, cudaMemsetAsync(grad_base, 0, sizeof(double) * n, ctx->stream));
        }
        return SOAPGB_OK;
    }
    double w01[2];
    if (host) {
        w01[0] = wave[0];
        w01[1] = wave[1];
    } else {
        SOAP_CUDA(ctx, cudaMemcpyAsync(w01, wave, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    const int wid = conv_halfwidth(w01[0], w01[1], sigma_v, window);
    if (wid < 1 || 2 * wid + 2 >= n)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_lower_resolution_adjoint: convolution half width %d invalid for n=%d",
                         wid, n);
    const size_t row_b = sizeof(double) * (size_t)n, spec_b = row_b * n_spec;
    const size_t out_b = sizeof(double) * (size_t)n_eff * n_spec;
    Workspace ws(ctx);
    int s_wave = ws.add(host ? row_b : 0);
    int s_base = ws.add(host && base ? row_b : 0);
    int s_spec = ws.add(host ? spec_b : 0);
    int s_g = ws.add(host ? out_b : 0);
    int s_gs = ws.add(host ? spec_b : 0);
    int s_gb = ws.add(host && grad_base ? row_b : 0);
    int s_conv = ws.add(out_b);
    int s_mm = ws.add(sizeof(unsigned long long) * 2 * n_spec);
    int s_kq = ws.add(sizeof(double) * n_eff), s_cq = ws.add(sizeof(double) * n_eff);
    int s_par = ws.add(sizeof(double) * 3 * n_spec), s_idx = ws.add(sizeof(int) * 2 * n_spec);
    int rc = ws.commit();
    if (rc) return rc;
    const double *d_wave = (const double *)stage_in(ctx, mem, wave, row_b, ws.get<void>(s_wave), &rc);
    if (rc) return rc;
    const double *d_base = (const double *)stage_in(ctx, mem, base, base ? row_b : 0, ws.get<void>(s_base), &rc);
    if (rc) return rc;
    const double *d_spec = (const double *)stage_in(ctx, mem, spec, spec_b, ws.get<void>(s_spec), &rc);
    if (rc) return rc;
    const double *d_g = (const double *)stage_in(ctx, mem, g_out, out_b, ws.get<void>(s_g), &rc);
    if (rc) return rc;
    double *d_gs = host ? ws.get<double>(s_gs) : grad_spec;
    double *d_gb = grad_base ? (host ? ws.get<double>(s_gb) : grad_base) : nullptr;
    double *conv = ws.get<double>(s_conv);
    unsigned long long *mm = ws.get<unsigned long long>(s_mm);
    double *kq = ws.get<double>(s_kq), *cq = ws.get<double>(s_cq), *par = ws.get<double>(s_par);
    int *idx = ws.get<int>(s_idx);
    // the forward's C and extrema, in the reference's operation order
    SOAP_TRACED(ctx, "conv_plain64",
                k_conv_plain64<<<dim3(grid_for(ctx, n_eff, 256), n_spec), 256, 0, ctx->stream>>>(
                    n, n_eff, d_wave, d_spec, n, d_base, nullptr, 0, sigma_v, wid, step_mult, step_exp, conv, n_eff));
    SOAP_LAUNCHED(ctx);
    k_minmax_init<<<(n_spec + 127) / 128, 128, 0, ctx->stream>>>(n_spec, sentinel, mm);
    SOAP_LAUNCHED(ctx);
    SOAP_TRACED(ctx, "minmax64",
                k_minmax<<<dim3(std::max(1, std::min(64, (n + 255) / 256)), n_spec), 256, 0, ctx->stream>>>(
                    n, n_eff, d_spec, n, d_base, nullptr, 0, conv, n_eff, nullptr, nullptr, mm));
    SOAP_LAUNCHED(ctx);
    k_radj_taps<<<grid_for(ctx, n_eff, 256), 256, 0, ctx->stream>>>(n, n_eff, d_wave, sigma_v, wid, step_mult,
                                                                     step_exp, kq, cq);
    SOAP_LAUNCHED(ctx);
    SOAP_TRACED(ctx, "resolution_adjoint_reduce",
                k_radj_reduce<<<n_spec, RADJ_THREADS, 0, ctx->stream>>>(n, n_eff, d_spec, d_base, conv, mm, d_g, par,
                                                                        idx));
    SOAP_LAUNCHED(ctx);
    SOAP_TRACED(ctx, "resolution_adjoint",
                k_radj_spec<<<dim3(grid_for(ctx, n, 256), n_spec), 256, 0, ctx->stream>>>(
                    n, n_eff, wid, kq, cq, d_g, par, idx, d_base ? 1 : 0, d_gs));
    SOAP_LAUNCHED(ctx);
    if (d_gb) {
        k_radj_base<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, n_spec, d_gs, d_gb);
        SOAP_LAUNCHED(ctx);
    }
    if (host) {
        SOAP_CUDA(ctx, cudaMemcpyAsync(grad_spec, d_gs, spec_b, cudaMemcpyDeviceToHost, ctx->stream));
        if (grad_base) SOAP_CUDA(ctx, cudaMemcpyAsync(grad_base, d_gb, row_b, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return check_status(ctx, "soapgb_lower_resolution_adjoint");
    }
    return SOAPGB_OK;
}
