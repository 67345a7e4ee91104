// Collapsed shift-FIR engine: the FAST64 / FAST32 forms of the disk and phase
// integration (the same function as SOAP_initialize.cu:339-395 and
// SOAP_integration.cu:392-447, re-associated).
//
// For a uniform wavelength grid the reference's per-cell interpolation at output
// pixel j reads the source position u_j = (j - off) / r (r = 1 + fbeta,
// off = fbeta lambda0 / step): owner i = floor(u_j), weight w = u_j - i.  Over a tile
// of T pixels starting at j0, u_j = i0 + dj + phi + delta dj with i0 = floor(u_{j0}),
// phi = u_{j0} - i0, delta = 1/r - 1 (|delta| ~ v/c ~ 1e-5).  While phi + delta dj
// stays in [0, 1) the cell contributes
//     L (1 - phi - delta dj) S_b[j - k] + L (phi + delta dj) S_b[j - k + 1],   k = j0 - i0,
// which is linear in dj with coefficients that only depend on (b, k).  Summing the
// coefficients of all such ("regular") cells per (kind, b, k) group collapses
// thousands of cells into a few dozen two-tap filters per tile; pixels whose owner
// j - k leaves [0, n_eff-2] are clipped per group.  Cells whose weight wraps inside
// the tile are added directly ("exceptions"), exactly as the per-cell form does.
//
// Per tile, a block of 256 threads owns 1024 pixels:
//   setup  -- position of every cell at j0 (FP64 in FAST64, float pairs in FAST32),
//             warp segmented reduction of equal keys (cells come in map order, so
//             keys repeat in runs), 64-bit fixed-point atomics into a shared hash;
//   apply  -- every thread walks the group list for its four pixels (coalesced
//             two-tap loads, compensated sums in FP32 for FAST32).
#include <algorithm>
#include <cmath>

#include "fir.cuh"

using namespace soapgb;

constexpr int FIR_THREADS = 256;
constexpr int FIR_PIX = 4;
constexpr int FIR_TILE = FIR_THREADS * FIR_PIX;
constexpr int FIR_HASH = 1024;     // shared hash slots (kind, bin, shift)
constexpr int FIR_EXC = 512;       // shared exception slots

enum { MODE_QUIET = 0, MODE_PHASE = 1 };

// per grid cell constants (phase independent)
struct CellGeo {
    double ir;     // 1 / (1 + fbeta)
    double offir;  // fbeta lambda0 / step / (1 + fbeta)
    double dlt;    // ir - 1
    double L;      // limb darkening
    double w2;     // (1 + LB) L
    // FP32 form: the position t(j0) = j0 dlt - offir in float pairs (hi + lo carries
    // 48 significant bits, the precision of the FP64 position), and FP32 weights
    float dlt_hi, dlt_lo, off_hi, off_lo;
    float Lf, w2f, dltf;
    int row;       // mu bin
    int zero_v;    // delta == 0: the reference copies the row
};

// the FP32 form's per-cell constants, two 16-byte loads:
// a = (dlt_hi, dlt_lo, off_hi, off_lo), b = (L, (1 + LB) L, dlt, bits(row | zero_v << 31))
struct __align__(16) CellGeo32 {
    float4 a, b;
};

// per (list, entry) record: x = grid cell, y = flags (bit 0 facula, bit 1 integral temperature)
__global__ void k_list_records(int n_lists, int max_cells, const int *__restrict__ cells,
                               const int *__restrict__ counts, const double *__restrict__ temp,
                               const double *__restrict__ bi, long long gm, int2 *recs) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int l = blockIdx.y;
    if (t >= counts[l]) return;
    int cell = cells[(long long)l * max_cells + t];
    int flags = 2;
    if (bi) {
        double b = bi[(long long)l * gm + cell];
        double tc = temp[(long long)l * gm + cell];
        flags = ((__double_as_longlong(b) << 1) == 0 ? 0 : 1);
        long long tb = __double_as_longlong(tc);
        int e = (int)((tb >> 52) & 0x7ff) - 1023;
        bool integral = (e >= 52) || (e < 0 ? (tb << 1) == 0 : ((tb & 0xfffffffffffffLL) & ((1LL << (52 - e)) - 1)) == 0);
        flags |= integral ? 2 : 0;
    }
    recs[(long long)l * max_cells + t] = make_int2(cell, flags);
}

__global__ void k_cell_geo(long long gm, const double *__restrict__ delta, const double *__restrict__ limb,
                           const double *__restrict__ lb, const int *__restrict__ region, int n_mu, double lambda0,
                           double step, CellGeo *geo, CellGeo32 *geo32, int *status) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= gm) return;
    double d = delta[k];
    CellGeo g;
    double beta = d * 1000. / SOAP_C_LIGHT;
    double fbeta = sqrt((1 + beta) / (1 - beta)) - 1;
    double r = 1 + fbeta;
    double off = fbeta * lambda0 / step;
    g.ir = 1.0 / r;
    g.offir = off / r;
    g.dlt = g.ir - 1.0;
    g.L = limb[k];
    g.w2 = lb ? (1.0 + lb[k]) * g.L : g.L;
    g.Lf = (float)g.L;
    g.w2f = (float)g.w2;
    g.dltf = (float)g.dlt;
    g.dlt_hi = (float)g.dlt;
    g.dlt_lo = (float)(g.dlt - (double)g.dlt_hi);
    g.off_hi = (float)g.offir;
    g.off_lo = (float)(g.offir - (double)g.off_hi);
    int row = region[k];
    if ((unsigned)row >= (unsigned)n_mu && g.L > -998.0) {
        atomicExch(status, 21);
        row = 0;
    }
    g.row = ((unsigned)row < (unsigned)n_mu) ? row : 0;
    g.zero_v = (d == 0.0);
    geo[k] = g;
    CellGeo32 h;
    h.a = make_float4(g.dlt_hi, g.dlt_lo, g.off_hi, g.off_lo);
    h.b = make_float4(g.Lf, g.w2f, g.dltf, __int_as_float(g.row | (g.zero_v ? (int)0x80000000 : 0)));
    geo32[k] = h;
}

// wavelength grid must be uniform for the collapsed form
__global__ void k_check_uniform(int n_eff, const double *__restrict__ lam, double step, int *status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_eff) return;
    double expect = lam[0] + (double)i * step;
    if (fabs(lam[i] - expect) > 1e-6 * step) atomicExch(status, 31);
}

template <typename T>
__global__ void k_to_type(long long count, const double *__restrict__ a, const double *__restrict__ b, T *out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    double v = b ? a[i] - b[i] : a[i];
    out[i] = (T)v;
}

// per-pixel sums of the FP32 form: compensated (Kahan) when set
constexpr bool FIR_COMPENSATED = true;

// per-pixel accumulator
template <typename T>
struct Acc {
    T s, c;
    __device__ __forceinline__ void zero() { s = (T)0; c = (T)0; }
    __device__ __forceinline__ void add(T x) {
        if constexpr (sizeof(T) == 4 && FIR_COMPENSATED) {
            T y = x - c;
            T t = s + y;
            c = (t - s) - y;
            s = t;
        } else {
            s += x;
        }
    }
    __device__ __forceinline__ double get() const { return (double)s - (double)c; }
};

// Source position of a cell at the tile start, on the FP32 pipe: u0 = j0 + t with
// t = j0 dlt - offir evaluated in float pairs (exact products by fmaf, TwoSum for
// the sums); returns i0 = floor(u0) and phi = u0 - i0.  |t| < 2^20 and j0 < 2^24.
__device__ __forceinline__ void fir_pos32(int j0, const float dlt_hi, const float dlt_lo, const float off_hi,
                                          const float off_lo, int &i0, float &phi) {
    float j0f = (float)j0;
    float pr = j0f * dlt_hi;
    float pe = fmaf(j0f, dlt_hi, -pr);
    float q = j0f * dlt_lo;
    float sm = pr - off_hi;
    float bp = sm - pr;
    float err = (pr - (sm - bp)) + (-off_hi - bp);
    float tl = err + (pe + (q - off_lo));
    float th = sm + tl;
    tl = tl - (th - sm);
    float fl = floorf(th);
    float fr = (th - fl) + tl;
    if (fr < 0.f) {
        fr += 1.f;
        fl -= 1.f;
    } else if (fr >= 1.f) {
        fr -= 1.f;
        fl += 1.f;
    }
    i0 = j0 + (int)fl;
    phi = fr;
}

// exact tests on FP64 values with integer instructions (no FP64 pipe)
__device__ __forceinline__ bool bits_is_zero(double v) { return (__double_as_longlong(v) << 1) == 0; }
__device__ __forceinline__ bool bits_is_integral(double v) {
    long long b = __double_as_longlong(v);
    int e = (int)((b >> 52) & 0x7ff) - 1023;
    if (e >= 52) return true;
    if (e < 0) return (b << 1) == 0;
    long long mant = b & 0xfffffffffffffLL;
    return (mant & ((1LL << (52 - e)) - 1)) == 0;
}

struct FirCubes {
    // PHASE: q_sed, q_norm, spot_norm, dq_spot, fac_norm, dq_fac; QUIET: [0] only
    const void *c[6];
    const double *spot_sed;
    const double *fac_sed;
    // FP32 form: the two continuum rows as float pairs (hi, lo)
    const float2 *spot_sed2;
    const float2 *fac_sed2;
};

template <typename T>
struct Exc {
    int i0;          // owner at j0
    int row;
    int kind;        // 0 spot, 1 facula (phase); 0 (quiet)
    int parts;       // 1: the L-weighted sums, 2: the (1+LB) L-weighted facula sums
    int zero_v;
    int plain_t;     // spot temperature is an integer: Planck ratio exactly 1
    T phi, dlt, L, w2;
    double temp;
};

__device__ __forceinline__ unsigned fir_key(int kind, int row, int k) {
    // kind < 4, row < 2^12, k in [-2^14, 2^14)
    return ((unsigned)kind << 28) | ((unsigned)row << 16) | (unsigned)((k + 16384) & 0xffff);
}

template <typename T>
__device__ __forceinline__ T lerp_at(const T *__restrict__ row, long long i, T w) {
    T s0 = row[i], s1 = row[i + 1];
    return s0 + (s1 - s0) * w;
}

// loi_Planck ratio B(lambda, t) / B(lambda, tn) (SOAP_integration.cu:205-212)
__device__ __forceinline__ double fir_planck_ratio(double lambda0, double t, double tn) {
    double c = 299792458.;
    double h = 6.62606896e-34;
    double k_b = 1.380e-23;
    double scale = 1e-10;
    double a = (h * c) / (lambda0 * k_b * scale);
    return (exp(a / tn) - 1) / (exp(a / t) - 1);
}

template <typename T>
struct FirShared {
    unsigned key[FIR_HASH];
    // group coefficients in 64-bit fixed point: integer atomics are native, exact and
    // order independent (A0, A1 scaled by 2^40, B by 2^56)
    unsigned long long val[FIR_HASH][3];
    int grp[FIR_HASH];
    float gcoef[FIR_HASH][3];   // FP32 form: group coefficients for the apply phase
    Exc<T> exc[FIR_EXC];
    int nexc, ngrp;
};

// float pair with an error term (TwoSum): the FP32 form's output combinations
struct F2 {
    float hi, lo;
};
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
    float s = a.hi + b.hi;
    float bp = s - a.hi;
    float e = (a.hi - (s - bp)) + (b.hi - bp);
    e += a.lo + b.lo;
    float hi = s + e;
    F2 r;
    r.hi = hi;
    r.lo = e - (hi - s);
    return r;
}

constexpr double FIX_A = 1099511627776.0;            // 2^40: A0, A1 (weights <= 1 per cell)
constexpr double FIX_B = 72057594037927936.0;        // 2^56: B (weight x delta, |delta| ~ 1e-5)
constexpr float FIX_A_F = 1099511627776.0f;
constexpr float FIX_B_F = 72057594037927936.0f;
__device__ __forceinline__ long long v_fix(double a, double scale) { return __double2ll_rn(a * scale); }
__device__ __forceinline__ long long v_fix(float a, float scale) {
    // a * 2^k is exact in FP32; the conversion rounds once
    return __float2ll_rn(a * scale);
}

// One pass of the warp-cooperative insertion: lanes holding a key (active) fold
// runs of equal keys (segmented scan of 64-bit fixed-point values: integer adds,
// exact and associative) and the run's last lane adds the sums to the shared hash
// table.  Returns whether this lane's contribution reached the table.
template <typename SH>
__device__ __forceinline__ bool fir_insert(SH &sh, bool active, unsigned key, long long a0, long long a1,
                                           long long bb, int lane) {
    if (!active) key = 0xfffffffeu;
    unsigned prev = __shfl_up_sync(0xffffffffu, key, 1);
    bool seg = (lane == 0) || (prev != key);
    // fast path: the whole warp is one run (cells come in map order, so most warps are)
    if (__all_sync(0xffffffffu, lane == 0 || !seg)) {
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) {
            a0 += __shfl_xor_sync(0xffffffffu, a0, o);
            a1 += __shfl_xor_sync(0xffffffffu, a1, o);
            bb += __shfl_xor_sync(0xffffffffu, bb, o);
        }
        bool ok = true;
        if (key != 0xfffffffeu && lane == 31) {
            ok = false;
            unsigned h = (key * 2654435761u) & (FIR_HASH - 1);
            for (int probe = 0; probe < 64 && !ok; ++probe) {
                unsigned old = atomicCAS(&sh.key[h], 0xffffffffu, key);
                if (old == 0xffffffffu || old == key) {
                    atomicAdd(&sh.val[h][0], (unsigned long long)a0);
                    atomicAdd(&sh.val[h][1], (unsigned long long)a1);
                    atomicAdd(&sh.val[h][2], (unsigned long long)bb);
                    ok = true;
                } else {
                    h = (h + 1) & (FIR_HASH - 1);
                }
            }
        }
        int all_ok = __shfl_sync(0xffffffffu, (int)ok, 31);
        return !active || all_ok;
    }
    for (int o = 1; o < 32; o <<= 1) {
        long long v0 = __shfl_up_sync(0xffffffffu, a0, o);
        long long v1 = __shfl_up_sync(0xffffffffu, a1, o);
        long long v2 = __shfl_up_sync(0xffffffffu, bb, o);
        int sg = __shfl_up_sync(0xffffffffu, (int)seg, o);
        if (lane >= o && !seg) {
            a0 += v0;
            a1 += v1;
            bb += v2;
            seg = sg;
        }
    }
    unsigned next = __shfl_down_sync(0xffffffffu, key, 1);
    bool tail = (lane == 31) || (next != key);
    bool ok = true;
    if (active && tail) {
        ok = false;
        unsigned h = (key * 2654435761u) & (FIR_HASH - 1);
        for (int probe = 0; probe < 64 && !ok; ++probe) {
            unsigned old = atomicCAS(&sh.key[h], 0xffffffffu, key);
            if (old == 0xffffffffu || old == key) {
                atomicAdd(&sh.val[h][0], (unsigned long long)a0);
                atomicAdd(&sh.val[h][1], (unsigned long long)a1);
                atomicAdd(&sh.val[h][2], (unsigned long long)bb);
                ok = true;
            } else {
                h = (h + 1) & (FIR_HASH - 1);
            }
        }
    }
    // every lane learns the outcome of its run's tail
    unsigned tails = __ballot_sync(0xffffffffu, tail);
    int my_tail = __ffs(tails & (0xffffffffu << lane)) - 1;
    int tail_ok = __shfl_sync(0xffffffffu, (int)ok, my_tail);
    return !active || tail_ok;
}

// a cell's three group coefficients in fixed point: A0 = w (1 - phi), A1 = w phi,
// B = w delta (the weight at pixel dj is A0 - B dj on the owner, A1 + B dj on owner + 1)
struct Coef3 {
    long long a0, a1, bb;
};
template <typename T>
__device__ __forceinline__ Coef3 coef3(T w, T phi, T dlt) {
    Coef3 r;
    if constexpr (sizeof(T) == 4) {
        r.a0 = v_fix(w * (1.0f - phi), FIX_A_F);
        r.a1 = v_fix(w * phi, FIX_A_F);
        r.bb = v_fix(w * dlt, FIX_B_F);
    } else {
        r.a0 = v_fix(w * (1.0 - phi), FIX_A);
        r.a1 = v_fix(w * phi, FIX_A);
        r.bb = v_fix(w * dlt, FIX_B);
    }
    return r;
}

// float-pair arithmetic for the FP32 form's output combination
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
    float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    float hi = p + e;
    F2 r;
    r.hi = hi;
    r.lo = e - (hi - p);
    return r;
}
__device__ __forceinline__ F2 f2_neg(F2 a) {
    a.hi = -a.hi;
    a.lo = -a.lo;
    return a;
}

// QUIET: OutT = double (one spectrum, once per star); PHASE: OutT = T (the FP32 form
// keeps its deficits in FP32 for the FP32 convolution that consumes them)
template <typename T, int MODE, typename OutT>
__global__ void __launch_bounds__(FIR_THREADS) k_fir(int n, int n_eff, const double *__restrict__ lam,
                                                     FirCubes cubes, const int2 *__restrict__ recs,
                                                     const int *__restrict__ counts, int max_cells,
                                                     const CellGeo *__restrict__ geo,
                                                     const CellGeo32 *__restrict__ geo32,
                                                     const double *__restrict__ temp, const double *__restrict__ bi,
                                                     long long gm, int solar, int t_norm_fac,
                                                     OutT *__restrict__ out0, OutT *__restrict__ out1,
                                                     OutT *__restrict__ out2, long long out_stride) {
    extern __shared__ __align__(16) unsigned char fir_smem[];
    FirShared<T> &sh = *reinterpret_cast<FirShared<T> *>(fir_smem);

    const int p = blockIdx.y;
    const int j0 = blockIdx.x * FIR_TILE;
    const int tid = threadIdx.x, lane = tid & 31;
    const int n_cells = counts[p];
    const int2 *pr = recs + (long long)p * max_cells;
    const double *pt = (MODE == MODE_PHASE) ? temp + (long long)p * gm : nullptr;
    const int t_eff = min(FIR_TILE, n_eff - j0);
    if (t_eff <= 0) {   // whole tile in the zero tail [n_eff, n)
        for (int q = 0; q < FIR_PIX; ++q) {
            int j = j0 + tid + q * FIR_THREADS;
            if (j >= n) continue;
            long long o = (long long)p * out_stride + j;
            out0[o] = (OutT)0;
            if constexpr (MODE == MODE_PHASE) { out1[o] = (OutT)0; out2[o] = (OutT)0; }
        }
        return;
    }

    for (int q = tid; q < FIR_HASH; q += FIR_THREADS) {
        sh.key[q] = 0xffffffffu;
        sh.val[q][0] = sh.val[q][1] = sh.val[q][2] = 0ULL;
    }
    if (tid == 0) sh.nexc = 0;

    // accumulators: QUIET [0]; PHASE: S, Qs, As, Bs, Qf, Af, Bf
    constexpr int NACC = (MODE == MODE_QUIET) ? 1 : 7;
    Acc<T> acc[NACC][FIR_PIX];
#pragma unroll
    for (int a = 0; a < NACC; ++a)
#pragma unroll
        for (int q = 0; q < FIR_PIX; ++q) acc[a][q].zero();
    __syncthreads();

    // direct evaluation of the collected exceptions (the per-cell arithmetic)
    auto flush = [&]() {
        int ne = sh.nexc;
        for (int e = 0; e < ne; ++e) {
            const Exc<T> &x = sh.exc[e];
            long long off = (long long)x.row * n;
#pragma unroll
            for (int q = 0; q < FIR_PIX; ++q) {
                int dj = tid + q * FIR_THREADS;
                int j = j0 + dj;
                if (j >= n_eff) continue;
                long long i;
                T w;
                if (x.zero_v) {
                    i = j;
                    w = (T)0;
                } else {
                    T wd = x.phi + x.dlt * (T)dj;
                    i = (long long)x.i0 + dj;
                    if (wd >= (T)1) { wd -= (T)1; i += 1; }
                    else if (wd < (T)0) { wd += (T)1; i -= 1; }
                    if (i < 0 || i > n_eff - 2) continue;
                    w = wd;
                }
                auto val = [&](int ci) -> T {
                    const T *rowp = reinterpret_cast<const T *>(cubes.c[ci]) + off;
                    if (x.zero_v) return rowp[i];
                    return lerp_at(rowp, i, w);
                };
                T L = x.L;
                if constexpr (MODE == MODE_QUIET) {
                    acc[0][q].add(L * val(0));
                } else {
                    if (x.parts & 1) {
                        acc[0][q].add(L * val(0));                              // S  (q_sed)
                        if (x.kind == 0) {
                            T Lq = L;
                            if (!x.plain_t)                                     // spot Planck ratio
                                Lq = (T)((double)x.L * fir_planck_ratio(lam[j], x.temp, (double)(int)x.temp));
                            acc[1][q].add(Lq * val(1));                         // Qs (q_norm)
                            acc[2][q].add(Lq * val(2));                         // As (spot_norm)
                            acc[3][q].add(L * val(3));                          // Bs (q_norm - spot_norm)
                        } else {
                            acc[6][q].add(L * val(5));                          // Bf (q_norm - fac_norm)
                        }
                    }
                    if ((x.parts & 2) && x.kind == 1) {
                        T w2 = x.w2;
                        if (solar) w2 = (T)((double)x.L * fir_planck_ratio(lam[j], x.temp, (double)t_norm_fac));
                        acc[4][q].add(w2 * val(1));                             // Qf
                        acc[5][q].add(w2 * val(4));                             // Af (fac_norm)
                    }
                }
            }
        }
    };

    // --- setup: place every cell at this tile -----------------------------------
    for (int c0 = 0; c0 < n_cells; c0 += FIR_THREADS) {
        int ci = c0 + tid;
        bool have = ci < n_cells;
        int2 rec = have ? pr[ci] : make_int2(0, 2);
        int cell = rec.x;
        int kind = (MODE == MODE_PHASE) ? (rec.y & 1) : 0;
        int plain_t = (rec.y >> 1) & 1;
        bool regular = false;
        int i0 = 0;
        T phi = (T)0, Lw, W2w, Dw;
        int row, zero_v;
        float dh = 0.f, dl = 0.f, oh = 0.f, ol = 0.f;
        double gir = 0.0, goff = 0.0;
        if constexpr (sizeof(T) == 4) {
            CellGeo32 h = geo32[cell];
            dh = h.a.x; dl = h.a.y; oh = h.a.z; ol = h.a.w;
            Lw = h.b.x; W2w = h.b.y; Dw = h.b.z;
            int rz = __float_as_int(h.b.w);
            row = rz & 0x7fffffff;
            zero_v = (rz >> 31) & 1;
        } else {
            const CellGeo &g = geo[cell];
            Lw = g.L; W2w = g.w2; Dw = g.dlt;
            row = g.row;
            zero_v = g.zero_v;
            gir = g.ir;
            goff = g.offir;
        }
        if (have) {
            if constexpr (sizeof(T) == 4) {
                float ph;
                fir_pos32(j0, dh, dl, oh, ol, i0, ph);
                phi = ph;
            } else {
                double u0 = fma((double)j0, gir, -goff);
                double fl = floor(u0);
                i0 = (int)fl;
                phi = u0 - fl;
            }
            // owners leaving [0, n_eff-2] do not break the linear form: the apply loop
            // clips each group's pixel range (pixels without an owner get nothing)
            T w_end = phi + Dw * (T)(t_eff - 1);
            int kk = j0 - i0;
            regular = (w_end >= (T)0) && (w_end < (T)1) && (kk >= -16384) && (kk < 16384);
            // v == 0 copies the row up to n_eff - 1, one pixel further than the clip
            if (zero_v) regular = regular && (j0 + t_eff - 1 <= n_eff - 2);
            if constexpr (MODE == MODE_PHASE) {
                if (kind == 0 && !plain_t) regular = false;    // spot Planck ratio != 1
                if (kind == 1 && solar) regular = false;       // per-pixel Planck ratio
            }
        }
        int k = j0 - i0;
        // pass A: weight L (spot: kind 0, facula: kind 1; quiet: kind 0)
        auto ca = coef3<T>(Lw, phi, Dw);
        bool okA = fir_insert(sh, have && regular, fir_key(kind, row, k), ca.a0, ca.a1, ca.bb, lane);
        bool okB = true;
        if constexpr (MODE == MODE_PHASE) {
            // pass B: facula (1 + LB) L weight
            auto cb = coef3<T>(W2w, phi, Dw);
            okB = fir_insert(sh, have && regular && kind == 1, fir_key(2, row, k), cb.a0, cb.a1, cb.bb, lane);
        }
        int parts = 0;
        if (have) {
            if (!regular) parts = 3;
            else parts = (okA ? 0 : 1) | (okB ? 0 : 2);
        }
        if (parts) {
            int slot = atomicAdd(&sh.nexc, 1);
            Exc<T> x;
            x.i0 = i0;
            x.row = row;
            x.kind = kind;
            x.parts = parts;
            x.zero_v = zero_v;
            x.plain_t = plain_t;
            x.phi = phi;
            x.dlt = Dw;
            x.L = Lw;
            x.w2 = W2w;
            x.temp = (MODE == MODE_PHASE && (!plain_t || solar)) ? pt[cell] : 0.0;
            sh.exc[slot] = x;
        }
        __syncthreads();
        if (sh.nexc > FIR_EXC - FIR_THREADS) {
            flush();
            __syncthreads();
            if (tid == 0) sh.nexc = 0;
        }
        __syncthreads();
    }
    flush();
    __syncthreads();
    // compact the occupied hash slots (ballot prefix per warp, warps in order)
    {
        constexpr int PER = FIR_HASH / FIR_THREADS;   // slots per thread
        static_assert(FIR_HASH % FIR_THREADS == 0, "hash size");
        int base_slot = tid * PER;
        int cnt = 0;
#pragma unroll
        for (int q = 0; q < PER; ++q) cnt += (sh.key[base_slot + q] != 0xffffffffu);
        int incl = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        __shared__ int wsum[FIR_THREADS / 32];
        if (lane == 31) wsum[tid >> 5] = incl;
        __syncthreads();
        int woff = 0;
        for (int w = 0; w < (tid >> 5); ++w) woff += wsum[w];
        int pos = woff + incl - cnt;
#pragma unroll
        for (int q = 0; q < PER; ++q)
            if (sh.key[base_slot + q] != 0xffffffffu) sh.grp[pos++] = base_slot + q;
        if (tid == FIR_THREADS - 1) sh.ngrp = woff + incl;
    }
    __syncthreads();
    for (int e = tid; e < sh.ngrp; e += FIR_THREADS) {
        int h = sh.grp[e];
        sh.gcoef[e][0] = __ll2float_rn((long long)sh.val[h][0]) * (1.0f / FIX_A_F);
        sh.gcoef[e][1] = __ll2float_rn((long long)sh.val[h][1]) * (1.0f / FIX_A_F);
        sh.gcoef[e][2] = __ll2float_rn((long long)sh.val[h][2]) * (1.0f / FIX_B_F);
    }
    __syncthreads();
    // --- apply the collapsed groups ---------------------------------------------
    int ng = sh.ngrp;
    for (int e = 0; e < ng; ++e) {
        int h = sh.grp[e];
        unsigned key = sh.key[h];
        int kind = (int)(key >> 28);
        int row = (int)((key >> 16) & 0xfff);
        int k = (int)(key & 0xffff) - 16384;
        T A0, A1, B;
        if constexpr (sizeof(T) == 4) {
            A0 = sh.gcoef[e][0];
            A1 = sh.gcoef[e][1];
            B = sh.gcoef[e][2];
        } else {
            A0 = __ll2double_rn((long long)sh.val[h][0]) * (1.0 / (double)FIX_A_F);
            A1 = __ll2double_rn((long long)sh.val[h][1]) * (1.0 / (double)FIX_A_F);
            B = __ll2double_rn((long long)sh.val[h][2]) * (1.0 / (double)FIX_B_F);
        }
        long long off = (long long)row * n;
        // pixels whose owner j - k lies in [0, n_eff - 2]
        const int jlo = max(j0, k);
        const int jhi = min(j0 + t_eff - 1, n_eff - 2 + k);
#pragma unroll
        for (int q = 0; q < FIR_PIX; ++q) {
            int dj = tid + q * FIR_THREADS;
            int j = j0 + dj;
            if (j < jlo || j > jhi) continue;
            long long i = (long long)j - k;
            T c0 = A0 - B * (T)dj;
            T c1 = A1 + B * (T)dj;
            auto two = [&](int ci) -> T {
                const T *rowp = reinterpret_cast<const T *>(cubes.c[ci]) + off;
                return c0 * rowp[i] + c1 * rowp[i + 1];
            };
            if constexpr (MODE == MODE_QUIET) {
                acc[0][q].add(two(0));
            } else {
                if (kind == 0) {              // spot, weight L
                    acc[0][q].add(two(0));
                    acc[1][q].add(two(1));
                    acc[2][q].add(two(2));
                    acc[3][q].add(two(3));
                } else if (kind == 1) {       // facula, weight L
                    acc[0][q].add(two(0));
                    acc[6][q].add(two(5));
                } else {                      // facula, weight (1 + LB) L
                    acc[4][q].add(two(1));
                    acc[5][q].add(two(4));
                }
            }
        }
    }
    // --- outputs ----------------------------------------------------------------
#pragma unroll
    for (int q = 0; q < FIR_PIX; ++q) {
        int j = j0 + tid + q * FIR_THREADS;
        if (j >= n) continue;
        long long o = (long long)p * out_stride + j;
        if (j >= n_eff) {
            out0[o] = (OutT)0;
            if constexpr (MODE == MODE_PHASE) { out1[o] = (OutT)0; out2[o] = (OutT)0; }
            continue;
        }
        if constexpr (MODE == MODE_QUIET) {
            out0[o] = (OutT)acc[0][q].get();
        } else if constexpr (sizeof(T) == 4) {
            // flux = S - I_s Qs - I_f Qf, tot = S - I_s As - I_f Af in float pairs: the
            // facula terms nearly cancel S, so no FP32 rounding before the subtraction
            F2 S{acc[0][q].s, -acc[0][q].c}, Qs{acc[1][q].s, -acc[1][q].c}, As{acc[2][q].s, -acc[2][q].c};
            F2 Qf{acc[4][q].s, -acc[4][q].c}, Af{acc[5][q].s, -acc[5][q].c};
            float2 is2 = cubes.spot_sed2[j], fs2 = cubes.fac_sed2[j];
            F2 is{is2.x, is2.y}, fs{fs2.x, fs2.y};
            F2 fl = f2_add(f2_add(S, f2_neg(f2_mul(is, Qs))), f2_neg(f2_mul(fs, Qf)));
            F2 tt = f2_add(f2_add(S, f2_neg(f2_mul(is, As))), f2_neg(f2_mul(fs, Af)));
            F2 bc = f2_add(F2{acc[3][q].s, -acc[3][q].c}, F2{acc[6][q].s, -acc[6][q].c});
            out0[o] = (OutT)(fl.hi + fl.lo);   // flux
            out1[o] = (OutT)(bc.hi + bc.lo);   // bconv
            out2[o] = (OutT)(tt.hi + tt.lo);   // tot
        } else {
            double S = acc[0][q].get(), Qs = acc[1][q].get(), As = acc[2][q].get(), Bs = acc[3][q].get();
            double Qf = acc[4][q].get(), Af = acc[5][q].get(), Bf = acc[6][q].get();
            double is = cubes.spot_sed[j], fs = cubes.fac_sed[j];
            out0[o] = (OutT)(S - is * Qs - fs * Qf);   // flux
            out1[o] = (OutT)(Bs + Bf);                 // bconv
            out2[o] = (OutT)(S - is * As - fs * Af);   // tot
        }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

__global__ void k_pair_rows(int n, const double *__restrict__ a, const double *__restrict__ b, float2 *pa, float2 *pb) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float ah = (float)a[i], bh = (float)b[i];
    pa[i] = make_float2(ah, (float)(a[i] - (double)ah));
    pb[i] = make_float2(bh, (float)(b[i] - (double)bh));
}

FirPlanSizes fir_plan_sizes(int form, int n, int n_mu, long long gm, bool phase, int n_lists) {
    FirPlanSizes p;
    if (form == SOAPGB_PLAIN64) return p;
    size_t tsz = (form == SOAPGB_FAST32) ? 4 : 8;
    size_t cube = align256(tsz * (size_t)n * n_mu);
    p.bytes = align256(sizeof(CellGeo) * (size_t)gm) + align256(sizeof(CellGeo32) * (size_t)gm) +
              (phase ? 6 : 1) * cube + 2 * align256(sizeof(float2) * n) +
              align256(sizeof(int2) * (size_t)gm * (size_t)(n_lists > 0 ? n_lists : 1));
    return p;
}

template <typename T, int MODE, typename OutT>
static int launch_fir(soapgb_ctx *ctx, int n, int n_eff, const double *lam, const FirCubes &fc, const int *cells,
                      const int *counts, int max_cells, const CellGeo *geo, const CellGeo32 *geo32, int2 *recs,
                      const double *temp, const double *bi, long long gm, int solar, int t_norm_fac, OutT *o0,
                      OutT *o1, OutT *o2, long long out_stride, int n_lists) {
    // records are written over the compacted cell lists, in place (int -> int2
    // needs its own buffer: recs)
    {
        dim3 gr(grid_for(ctx, max_cells, 256), n_lists);
        k_list_records<<<gr, 256, 0, ctx->stream>>>(n_lists, max_cells, cells, counts, temp, bi, gm, recs);
        SOAP_LAUNCHED(ctx);
    }
    size_t smem = sizeof(FirShared<T>);
    SOAP_CUDA(ctx, cudaFuncSetAttribute(k_fir<T, MODE, OutT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // tiles cover [0, n): tiles past n_eff only write the zero tail
    dim3 g((n + FIR_TILE - 1) / FIR_TILE, n_lists);
    k_fir<T, MODE, OutT><<<g, FIR_THREADS, smem, ctx->stream>>>(n, n_eff, lam, fc, recs, counts, max_cells, geo,
                                                                geo32, temp, bi, gm, solar, t_norm_fac, o0, o1, o2,
                                                                out_stride);
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}

static int fir_prepare(soapgb_ctx *ctx, const double *wave, int n_eff, double step, long long gm, const double *delta,
                       const double *limb, const double *lb, const int *region, int n_mu, CellGeo *geo,
                       CellGeo32 *geo32) {
    double lambda0;
    SOAP_CUDA(ctx, cudaMemcpyAsync(&lambda0, wave, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    k_check_uniform<<<grid_for(ctx, n_eff, 256), 256, 0, ctx->stream>>>(n_eff, wave, step, ctx->d_status);
    SOAP_LAUNCHED(ctx);
    k_cell_geo<<<grid_for(ctx, gm, 256), 256, 0, ctx->stream>>>(gm, delta, limb, lb, region, n_mu, lambda0, step, geo,
                                                                geo32, ctx->d_status);
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}

int fir_quiet(soapgb_ctx *ctx, int form, const FirQuietArgs &a, char *scratch, const FirPlanSizes &plan) {
    (void)plan;
    size_t tsz = (form == SOAPGB_FAST32) ? 4 : 8;
    size_t cube_elems = (size_t)a.n * a.n_mu;
    long long gm = a.max_cells;
    char *p = scratch;
    CellGeo *geo = (CellGeo *)p;
    p += align256(sizeof(CellGeo) * (size_t)gm);
    CellGeo32 *geo32 = (CellGeo32 *)p;
    p += align256(sizeof(CellGeo32) * (size_t)gm);
    void *cube = p;
    p += align256(tsz * cube_elems);
    int2 *recs = (int2 *)p;
    p += align256(sizeof(int2) * (size_t)gm);
    int rc = fir_prepare(ctx, a.wave, a.n_eff, a.step, gm, a.delta, a.limb, nullptr, a.region, a.n_mu, geo, geo32);
    if (rc) return rc;
    FirCubes fc{};
    if (form == SOAPGB_FAST32) {
        k_to_type<float><<<grid_for(ctx, cube_elems, 256), 256, 0, ctx->stream>>>(cube_elems, a.cube, nullptr, (float *)cube);
        SOAP_LAUNCHED(ctx);
        fc.c[0] = cube;
        return launch_fir<float, MODE_QUIET, double>(ctx, a.n, a.n_eff, a.wave, fc, a.cells, a.n_cells, a.max_cells,
                                                     geo, geo32, recs, nullptr, nullptr, gm, 0, 0, a.out, nullptr,
                                                     nullptr, 0, 1);
    }
    fc.c[0] = a.cube;
    return launch_fir<double, MODE_QUIET, double>(ctx, a.n, a.n_eff, a.wave, fc, a.cells, a.n_cells, a.max_cells, geo,
                                                  geo32, recs, nullptr, nullptr, gm, 0, 0, a.out, nullptr, nullptr, 0,
                                                  1);
}

int fir_phase(soapgb_ctx *ctx, int form, const FirPhaseArgs &a, char *scratch, const FirPlanSizes &plan) {
    (void)plan;
    size_t tsz = (form == SOAPGB_FAST32) ? 4 : 8;
    int n_mu = a.cubes->n_mu;
    size_t cube_elems = (size_t)a.n * n_mu;
    char *p = scratch;
    CellGeo *geo = (CellGeo *)p;
    p += align256(sizeof(CellGeo) * (size_t)a.gm);
    CellGeo32 *geo32 = (CellGeo32 *)p;
    p += align256(sizeof(CellGeo32) * (size_t)a.gm);
    int2 *recs = (int2 *)p;
    p += align256(sizeof(int2) * (size_t)a.gm * (size_t)a.n_phase);
    void *cb[6];
    for (int q = 0; q < 6; ++q) {
        cb[q] = p;
        p += align256(tsz * cube_elems);
    }
    float2 *sed2a = (float2 *)p;
    p += align256(sizeof(float2) * a.n);
    float2 *sed2b = (float2 *)p;
    int rc = fir_prepare(ctx, a.wave, a.n_eff, a.step, a.gm, a.delta, a.limb, a.lb, a.region, n_mu, geo, geo32);
    if (rc) return rc;
    const soapgb_cubes &c = *a.cubes;
    // typed cubes: q_sed, q_norm, spot_norm, q_norm - spot_norm, fac_norm, q_norm - fac_norm
    const double *src_a[6] = {c.q_sed, c.q_norm, c.spot_norm, c.q_norm, c.fac_norm, c.q_norm};
    const double *src_b[6] = {nullptr, nullptr, nullptr, c.spot_norm, nullptr, c.fac_norm};
    FirCubes fc{};
    for (int q = 0; q < 6; ++q) {
        if (form == SOAPGB_FAST32)
            k_to_type<float><<<grid_for(ctx, cube_elems, 256), 256, 0, ctx->stream>>>(cube_elems, src_a[q], src_b[q], (float *)cb[q]);
        else
            k_to_type<double><<<grid_for(ctx, cube_elems, 256), 256, 0, ctx->stream>>>(cube_elems, src_a[q], src_b[q], (double *)cb[q]);
        SOAP_LAUNCHED(ctx);
        fc.c[q] = cb[q];
    }
    fc.spot_sed = c.spot_sed;
    fc.fac_sed = c.fac_sed;
    int t_norm_fac = (int)(a.act->t_star + a.act->t_diff_fac + 0.9 - 216.8);
    if (form == SOAPGB_FAST32) {
        k_pair_rows<<<grid_for(ctx, a.n, 256), 256, 0, ctx->stream>>>(a.n, c.spot_sed, c.fac_sed, sed2a, sed2b);
        SOAP_LAUNCHED(ctx);
        fc.spot_sed2 = sed2a;
        fc.fac_sed2 = sed2b;
        if (!a.out_f32) return set_error(ctx, SOAPGB_ERR_ARG, "FP32 form writes FP32 deficits");
        return launch_fir<float, MODE_PHASE, float>(ctx, a.n, a.n_eff, a.wave, fc, a.cells, a.counts, a.max_cells,
                                                    geo, geo32, recs, a.temp, a.bi, a.gm, a.act->solar, t_norm_fac,
                                                    (float *)a.flux, (float *)a.bconv, (float *)a.tot, a.out_stride,
                                                    a.n_phase);
    }
    if (a.out_f32) return set_error(ctx, SOAPGB_ERR_ARG, "FP64 form writes FP64 deficits");
    return launch_fir<double, MODE_PHASE, double>(ctx, a.n, a.n_eff, a.wave, fc, a.cells, a.counts, a.max_cells, geo,
                                                  geo32, recs, a.temp, a.bi, a.gm, a.act->solar, t_norm_fac,
                                                  (double *)a.flux,
                                                  (double *)a.bconv, (double *)a.tot, a.out_stride, a.n_phase);
}
