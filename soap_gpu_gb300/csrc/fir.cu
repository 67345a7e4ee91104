// Collapsed shift-FIR engine: the FAST64 / FAST32 forms of the disk and phase
// integration (the same function as SOAP_initialize.cu:339-395 and
// SOAP_integration.cu:392-447, re-associated).
//
// For a uniform wavelength grid the reference's per-cell interpolation at output
// pixel j reads the source position u_j = (j - off) / r (r = 1 + fbeta,
// off = fbeta lambda0 / step): owner i = floor(u_j), weight w = u_j - i.  Write
// u_j = j + t_c(j) with t_c(j) = j dlt_c - offir_c = dlt_c (j + lambda0 / step),
// dlt = 1/r - 1 (|dlt| ~ v/c ~ 1e-5).  Over a tile of T pixels from j0, a cell whose
// m = floor(t_c) does not change inside the tile contributes
//     L (1 - phi - dlt dj) S_b[j + m] + L (phi + dlt dj) S_b[j + m + 1],   phi = t_c(j0) - m,
// which is linear in dj; its coefficients summed over all cells sharing (b, m) are
//     A1 = sum L phi = j0 sum(L dlt) - sum(L offir) - m sum L,  A0 = sum L - A1,  B = sum L dlt.
// Cells sorted by (mu bin b, v == 0, dlt) have t_c(j) increasing with dlt at every j,
// so the cells of one (b, m) group form a contiguous range in that order: a tile
// finds each range with two binary searches and takes its coefficients from FP64
// prefix sums -- no per-cell work for the regular cells.  Cells whose m changes
// inside the tile ("wrap" cells, ~|dlt| T of them) lie between consecutive ranges
// and are evaluated directly, as are spots of non-integral temperature and the
// solar variant's faculae (per-pixel Planck ratio).  Pixels whose owner j + m leaves
// [0, n_eff - 2] get nothing from the group, as in the per-cell form.
//
// Per tile of 1024 pixels, a block of 256 threads walks its list's (class, mu bin)
// segments in work units of at most FIR_MCH shift values.  Each unit's source
// windows -- up to four cube rows, 1024 + (shift span) + 2 values each -- are staged
// in shared memory by TMA bulk copies (cp.async.bulk, mbarrier completion), double
// buffered so that the next unit's rows arrive while the current one is applied.
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "fir.cuh"
#include "regions.cuh"

using namespace soapgb;

constexpr int FIR_THREADS = 256;
constexpr int FIR_WARPS = FIR_THREADS / 32;
constexpr int FIR_PIX = 4;
constexpr int FIR_TILE = FIR_THREADS * FIR_PIX;
constexpr int FIR_WIN = 1152;                    // staged values per cube row (window capacity)
constexpr int FIR_MCH = FIR_WIN - FIR_TILE - 8;  // shift values per work unit (window + alignment fit)
constexpr int FIR_EXC = 256;                     // exceptions per batch
constexpr int FIR_MAX_MU = 256;
constexpr long long FIR_WAIT_LIMIT = 1LL << 24;  // bounded mbarrier waits

static_assert(FIR_MCH <= FIR_THREADS, "one shift value per thread in a unit");

// four rows of one class interleaved per pixel (the rows a work unit stages): one bulk
// copy stages a unit's window, one 16-byte (FP32) shared load fetches a pixel's 4 values
struct __align__(32) soap_double4 {
    double x, y, z, w;
};
template <typename T> struct Vec4T;
template <> struct Vec4T<float> { using type = float4; };
template <> struct Vec4T<double> { using type = soap_double4; };
template <typename T> using Vec4 = typename Vec4T<T>::type;


enum { MODE_QUIET = 0, MODE_PHASE = 1 };
enum { CLS_SPOT = 0, CLS_FAC = 1, CLS_DIRECT = 2 };

// status words written by the kernels of this file
enum { FIR_ST_UNIFORM = 31, FIR_ST_SEGMENTS = 34, FIR_ST_FAST = 35, FIR_ST_WAIT = 41 };

// per grid cell constants (phase independent)
struct CellGeo {
    double ir;     // 1 / (1 + fbeta)
    double offir;  // fbeta lambda0 / step / (1 + fbeta)
    double dlt;    // ir - 1
    double L;      // limb darkening
    double w2;     // (1 + LB) L
    int row;       // mu bin
    int zero_v;    // delta == 0: the reference copies the row
};

// the FP32 form's per-cell constants, two 16-byte loads:
// a = (dlt_hi, dlt_lo, offir_hi, offir_lo) (t(j0) = j0 dlt - offir in float pairs, the
// 48 significant bits of the FP64 position), b = (L, (1 + LB) L, dlt, bits(row | zero_v << 31))
struct __align__(16) CellGeo32 {
    float4 a, b;
};

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
    int row = region[k];
    bool visible = g.L > -998.0;
    if ((unsigned)row >= (unsigned)n_mu && visible) {
        atomicExch(status, 21);
        row = 0;
    }
    g.row = ((unsigned)row < (unsigned)n_mu) ? row : 0;
    g.zero_v = (d == 0.0);
    geo[k] = g;
    CellGeo32 h;
    float dh = (float)g.dlt, oh = (float)g.offir;
    h.a = make_float4(dh, (float)(g.dlt - (double)dh), oh, (float)(g.offir - (double)oh));
    h.b = make_float4((float)g.L, (float)g.w2, (float)g.dlt, __int_as_float(g.row | (g.zero_v ? (int)0x80000000 : 0)));
    geo32[k] = h;
}

// wavelength grid must be uniform for the collapsed form
__global__ void k_check_uniform(int n_eff, const double *__restrict__ lam, double step, int *status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_eff) return;
    double expect = lam[0] + (double)i * step;
    if (fabs(lam[i] - expect) > 1e-6 * step) atomicExch(status, FIR_ST_UNIFORM);
}

template <typename T>
__global__ void k_to_type(long long count, const double *__restrict__ a, const double *__restrict__ b, T *out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    double v = b ? a[i] - b[i] : a[i];
    out[i] = (T)v;
}

// FP64 -> FP32 rounded to nearest even on the integer pipes: the 52-bit fraction is cut
// to 23 bits, rounding up past half and at half to even (a carry into the exponent is
// the correct next binade, and past the largest exponent gives infinity).  Results
// outside the normal FP32 range (zero, subnormal) and NaN take the conversion
// instruction.
__device__ __forceinline__ float soap_f64_to_f32(double v) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((u >> 52) & 0x7ff);
    if (e < 1023 - 126 || e > 1023 + 127) return __double2float_rn(v);
    const unsigned long long frac = u & 0xfffffffffffffULL;
    const unsigned keep = (unsigned)(frac >> 29);
    const unsigned long long rest = frac & 0x1fffffffULL;
    unsigned bits = ((unsigned)(e - 1023 + 127) << 23) | keep;
    if (rest > 0x10000000ULL || (rest == 0x10000000ULL && (keep & 1u))) bits += 1u;
    return __uint_as_float(bits | ((unsigned)(u >> 32) & 0x80000000u));
}

// int -> FP64, exact, on the integer pipes (the conversion instruction runs on GB300's
// FP64 pipe, at 1/64 of the FP32 rate)
__device__ __forceinline__ double soap_i2d(int m) {
    if (m == 0) return 0.0;
    const unsigned long long s = m < 0 ? 1ull : 0ull;
    const unsigned a = m < 0 ? 0u - (unsigned)m : (unsigned)m;
    const int e = 31 - __clz((int)a);   // a in [2^e, 2^(e+1))
    const unsigned long long frac = ((unsigned long long)a << (52 - e)) & 0xfffffffffffffULL;
    return __longlong_as_double((long long)((s << 63) | ((unsigned long long)(1023 + e) << 52) | frac));
}
// FP64 -> T rounded to nearest (FP32: on the integer pipes)
template <typename T>
__device__ __forceinline__ T soap_to(double v) {
    if constexpr (sizeof(T) == 4) return soap_f64_to_f32(v);
    else return v;
}

// The interleaved rows of the two classes in one pass over the four FP64 cubes, pixel
// pairs per thread: spot (q_sed, q_norm, spot_norm, q_norm - spot_norm) and facula
// (q_sed, q_norm - fac_norm, q_norm, fac_norm), the differences formed in FP64 and
// rounded once.  Each thread keeps two steps' loads (eight 16-byte loads) in flight.
__device__ __forceinline__ void cube_rows_store(long long i, double2 a, double2 b, double2 c, double2 d, float4 *sp,
                                                float4 *fa) {
    const float qs0 = soap_f64_to_f32(a.x), qs1 = soap_f64_to_f32(a.y);
    const float qn0 = soap_f64_to_f32(b.x), qn1 = soap_f64_to_f32(b.y);
    sp[2 * i] = make_float4(qs0, qn0, soap_f64_to_f32(c.x), soap_f64_to_f32(b.x - c.x));
    sp[2 * i + 1] = make_float4(qs1, qn1, soap_f64_to_f32(c.y), soap_f64_to_f32(b.y - c.y));
    fa[2 * i] = make_float4(qs0, soap_f64_to_f32(b.x - d.x), qn0, soap_f64_to_f32(d.x));
    fa[2 * i + 1] = make_float4(qs1, soap_f64_to_f32(b.y - d.y), qn1, soap_f64_to_f32(d.y));
}

__global__ void __launch_bounds__(256) k_cube_types32(long long n2, const double2 *__restrict__ qs,
                                                      const double2 *__restrict__ qn, const double2 *__restrict__ sn,
                                                      const double2 *__restrict__ fn, float4 *sp, float4 *fa) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += 2 * stride) {
        const long long j = i + stride;
        const double2 a0 = __ldcs(qs + i), b0 = __ldcs(qn + i), c0 = __ldcs(sn + i), d0 = __ldcs(fn + i);
        double2 a1 = make_double2(0.0, 0.0), b1 = a1, c1 = a1, d1 = a1;
        if (j < n2) {
            a1 = __ldcs(qs + j);
            b1 = __ldcs(qn + j);
            c1 = __ldcs(sn + j);
            d1 = __ldcs(fn + j);
        }
        cube_rows_store(i, a0, b0, c0, d0, sp, fa);
        if (j < n2) cube_rows_store(j, a1, b1, c1, d1, sp, fa);
    }
}

// the same interleaved rows of any element type, one pixel per thread (the FP64 form, and
// cubes whose layout the paired kernel cannot take)
template <typename T>
__global__ void k_cube_rows(long long count, const double *__restrict__ qs, const double *__restrict__ qn,
                            const double *__restrict__ sn, const double *__restrict__ fn, Vec4<T> *sp, Vec4<T> *fa) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const double a = qs[i], b = qn[i], c = sn[i], d = fn[i];
    Vec4<T> s, f;
    s.x = (T)a;
    s.y = (T)b;
    s.z = (T)c;
    s.w = (T)(b - c);
    f.x = (T)a;
    f.y = (T)(b - d);
    f.z = (T)b;
    f.w = (T)d;
    sp[i] = s;
    fa[i] = f;
}

// --- cell order ----------------------------------------------------------------
// pass 1 keys: the slope dlt (order-preserving 64-bit image); pass 2 (stable): mu bin
// and v == 0, invisible cells last
__global__ void k_sort_keys1(long long gm, const CellGeo *__restrict__ geo, unsigned long long *keys, int *vals) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= gm) return;
    keys[k] = soap_ord64(geo[k].dlt);
    vals[k] = (int)k;
}

__global__ void k_sort_keys2(long long gm, const CellGeo *__restrict__ geo, const int *__restrict__ order,
                             unsigned *keys) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= gm) return;
    const CellGeo &g = geo[order[k]];
    keys[k] = (g.L > -998.0) ? (unsigned)(g.row * 2 + g.zero_v) : 0x3fffu;
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

// --- per-list cell lists in velocity order ---------------------------------------
// One block per list (the quiet disk, or one phase): the visible cells in the sorted
// order, split into classes -- 0: spots (integral temperature, Planck ratio exactly 1),
// 1: faculae, 2: cells evaluated directly (other spots; faculae of the solar
// variant).  counts[l] = (n0, n1, n2, 0); class c occupies positions
// [n0 + .. + n_{c-1}, + n_c) of the list.  Active cells are those whose type map value
// lies in [-0.5, 1.5] (0 spot, otherwise facula), as in the per-cell form's compaction.
// class of a visible cell of temperature t and type b (-1: not active)
__device__ __forceinline__ int fir_class_tb(const CellGeo &g, double t, double b, int solar) {
    if (!(g.L > -998.0)) return -1;
    if (!(b >= -0.5 && b <= 1.5)) return -1;
    if (bits_is_zero(b)) return bits_is_integral(t) ? CLS_SPOT : CLS_DIRECT;
    return solar ? CLS_DIRECT : CLS_FAC;
}

// fir_class_tb for a box cell of a region of type `type` (b = 0 or 1; a spot's
// temperature t_star - t_diff_spot is integral), with no FP64 instruction: the limb
// test !(L > -998) on the order-preserving integer images (a NaN is not visible)
__device__ __forceinline__ int fir_class_box(const CellGeo &g, int type, int solar) {
    const unsigned long long lb = (unsigned long long)__double_as_longlong(g.L);
    if ((lb & 0x7fffffffffffffffULL) > 0x7ff0000000000000ULL) return -1;   // NaN
    if (!(soap_ord64(g.L) > soap_ord64(-998.0))) return -1;
    if (type == 0) return CLS_SPOT;
    return solar ? CLS_DIRECT : CLS_FAC;
}

__device__ __forceinline__ int fir_class(const CellGeo &g, const double *bi, const double *temp, long long idx,
                                         int solar) {
    if (!(g.L > -998.0)) return -1;
    if (!bi) return CLS_SPOT;
    const double b = bi[idx];
    if (!(b >= -0.5 && b <= 1.5)) return -1;
    return fir_class_tb(g, bits_is_zero(b) ? temp[idx] : 0.0, b, solar);
}

__global__ void __launch_bounds__(1024) k_fir_lists(long long gm, const int *__restrict__ order,
                                                    const CellGeo *__restrict__ geo, const double *__restrict__ temp,
                                                    const double *__restrict__ bi, int solar, int *list_cell,
                                                    double *list_dlt, double2 *list_aux, int *counts,
                                                    int only_flagged) {
    const int l = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (only_flagged && counts[4 * l + 3] == 0) return;   // list already built by k_fir_plists
    const int nw = blockDim.x >> 5;
    const long long mbase = (long long)l * gm;
    __shared__ int cnt[3];
    __shared__ int wc[32][3];
    __shared__ int base[3];
    if (tid < 3) cnt[tid] = 0;
    __syncthreads();
    int my[3] = {0, 0, 0};
    for (long long r = tid; r < gm; r += blockDim.x) {
        int cell = order[r];
        int c = fir_class(geo[cell], bi, temp, mbase + cell, solar);
        if (c >= 0) my[c]++;
    }
    for (int c = 0; c < 3; ++c) {
        int v = my[c];
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) atomicAdd(&cnt[c], v);
    }
    __syncthreads();
    if (tid == 0) {
        base[0] = 0;
        base[1] = cnt[0];
        base[2] = cnt[0] + cnt[1];
        int *o = counts + 4 * l;
        o[0] = cnt[0];
        o[1] = cnt[1];
        o[2] = cnt[2];
        o[3] = 0;
    }
    __syncthreads();
    // ordered compaction, blockDim entries per pass
    for (long long r0 = 0; r0 < gm; r0 += blockDim.x) {
        long long r = r0 + tid;
        int c = -1, cell = 0;
        double d = 0.0;
        if (r < gm) {
            cell = order[r];
            const CellGeo &g = geo[cell];
            c = fir_class(g, bi, temp, mbase + cell, solar);
            d = g.dlt;
        }
        unsigned m[3];
        for (int q = 0; q < 3; ++q) m[q] = __ballot_sync(0xffffffffu, c == q);
        if (lane == 0)
            for (int q = 0; q < 3; ++q) wc[warp][q] = __popc(m[q]);
        __syncthreads();
        if (c >= 0) {
            int pos = base[c] + __popc(m[c] & ((1u << lane) - 1));
            for (int w = 0; w < warp; ++w) pos += wc[w][c];
            list_cell[mbase + pos] = cell;
            list_dlt[mbase + pos] = d;
            if (c == CLS_DIRECT) list_aux[mbase + pos] = make_double2(temp[mbase + cell], bi[mbase + cell]);
        }
        __syncthreads();
        if (tid < 3) {
            int s = 0;
            for (int w = 0; w < nw; ++w) s += wc[w][tid];
            base[tid] += s;
        }
        __syncthreads();
    }
}

// inverse of the cell order: rank[order[r]] = r
__global__ void k_fir_rank(long long gm, const int *__restrict__ order, int *rank) {
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < gm) rank[order[r]] = (int)r;
}

// Phase lists of at most FIR_PLIST_CAP active cells (the usual case): one block per
// phase scans the type map (coalesced), collects (class, rank) keys of the active cells
// in shared memory and sorts them (bitonic), which gives the same lists as k_fir_lists
// without visiting every visible cell per phase.  Longer lists are flagged
// (counts[4l + 3] = 1) and built by k_fir_lists.
constexpr int FIR_PLIST_CAP = 4096;

__global__ void __launch_bounds__(512) k_fir_plists(long long gm, const int *__restrict__ order,
                                                   const int *__restrict__ rank, const CellGeo *__restrict__ geo,
                                                   const double *__restrict__ temp, const double *__restrict__ bi,
                                                   int solar, int *list_cell, double *list_dlt, double2 *list_aux,
                                                   int *counts) {
    __shared__ unsigned keys[FIR_PLIST_CAP];
    __shared__ int cnt[4];
    const int l = blockIdx.x, tid = threadIdx.x;
    const long long mbase = (long long)l * gm;
    if (tid < 4) cnt[tid] = 0;
    __syncthreads();
    for (long long k = tid; k < gm; k += blockDim.x) {
        const double b = bi[mbase + k];
        if (!(b >= -0.5 && b <= 1.5)) continue;
        const int c = fir_class(geo[k], bi, temp, mbase + k, solar);
        if (c < 0) continue;
        atomicAdd(&cnt[c + 1], 1);
        const int pos = atomicAdd(&cnt[0], 1);
        if (pos < FIR_PLIST_CAP) keys[pos] = ((unsigned)c << 24) | (unsigned)rank[k];
    }
    __syncthreads();
    const int n = cnt[0];
    if (n > FIR_PLIST_CAP) {
        if (tid == 0) counts[4 * l + 3] = 1;
        return;
    }
    int np = 1;
    while (np < n) np <<= 1;
    for (int i = n + tid; i < np; i += blockDim.x) keys[i] = 0xffffffffu;
    __syncthreads();
    for (int k = 2; k <= np; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < np; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const unsigned a = keys[i], b2 = keys[ixj];
                    const bool up = ((i & k) == 0);
                    if ((a > b2) == up) {
                        keys[i] = b2;
                        keys[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = tid; i < n; i += blockDim.x) {
        const int cell = order[keys[i] & 0xffffffu];
        list_cell[mbase + i] = cell;
        list_dlt[mbase + i] = geo[cell].dlt;
        if ((int)(keys[i] >> 24) == CLS_DIRECT) list_aux[mbase + i] = make_double2(temp[mbase + cell], bi[mbase + cell]);
    }
    if (tid == 0) {
        int *o = counts + 4 * l;
        o[0] = cnt[1];
        o[1] = cnt[2];
        o[2] = cnt[3];
        o[3] = 0;
    }
}

// Phase lists without maps (the pipeline's collapsed forms): one block per phase visits
// the cells of its regions' bounding boxes only -- a few thousand of the G*G -- and
// keeps a cell in the box of the region that sets its final value (the last covering
// one, region_cell_value), so every active cell is found once.  The active cells are
// marked in three bitmaps over the velocity order (one per class) in shared memory; an
// ordered compaction of the bitmaps gives the same lists as k_fir_lists / k_fir_plists
// on the maps of k_phase_scan, with no sort and no G*G map per phase.
constexpr int FIR_BLIST_THREADS = 1024;
constexpr size_t FIR_BLIST_SMEM_MAX = 180 * 1024;

__global__ void __launch_bounds__(FIR_BLIST_THREADS)
    k_fir_blists(int grid, double delta_grid, const RegionPhase *__restrict__ table, const int *__restrict__ reg_off,
                 int t_star, int t_diff_spot, int t_diff_fac, int solar, const int *__restrict__ order,
                 const int *__restrict__ rank, const CellGeo *__restrict__ geo, int *list_cell, double *list_dlt,
                 double2 *list_aux, int *counts) {
    extern __shared__ unsigned bm[];   // [class][W] bitmaps over the velocity order
    __shared__ int wsum[FIR_BLIST_THREADS / 32];
    __shared__ int ctot[3];
    const long long gm = (long long)grid * grid;
    const int W = (int)((gm + 31) >> 5);
    const int l = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long mbase = (long long)l * gm;
    for (int i = tid; i < 3 * W; i += FIR_BLIST_THREADS) bm[i] = 0u;
    if (tid < 3) ctot[tid] = 0;
    __syncthreads();
    const int r0 = reg_off[l], r1 = reg_off[l + 1];
    const float delta_f = (float)delta_grid;
    for (int r = r0; r < r1; ++r) {
        const RegionPhase rp = table[r];
        const int by = rp.iy1 - rp.iy0, bz = rp.iz1 - rp.iz0;
        if (!rp.visible || by <= 0 || bz <= 0) continue;
        const int nbox = by * bz;
        for (int q = tid; q < nbox; q += FIR_BLIST_THREADS) {
            const int iy = rp.iy0 + q / bz, iz = rp.iz0 + q % bz;
            int owner = region_owner_fp32(table, r0, r1, iy, iz, delta_f);
            if (owner == -2) {
                double t, b;
                owner = region_cell_value(table, r0, r1, iy, iz, delta_grid, t_star, t_diff_spot, t_diff_fac, t, b);
            }
            if (owner != r) continue;
            // the class needs the type alone: a spot's temperature t_star - t_diff_spot is
            // integral, a facula's class does not depend on its temperature
            const int k = iy * grid + iz;
            const int c = fir_class_box(geo[k], rp.type, solar);
            if (c < 0) continue;
            const int rk = rank[k];
            atomicOr(&bm[c * W + (rk >> 5)], 1u << (rk & 31));
        }
    }
    __syncthreads();
    // ordered compaction: thread tid owns words [w0, w1) of the concatenated bitmaps
    const int nw3 = 3 * W;
    const int per = (nw3 + FIR_BLIST_THREADS - 1) / FIR_BLIST_THREADS;
    const int w0 = min(nw3, tid * per), w1 = min(nw3, w0 + per);
    int my = 0, myc[3] = {0, 0, 0};
    for (int w = w0; w < w1; ++w) {
        const int pc = __popc(bm[w]);
        my += pc;
        myc[w / W] += pc;
    }
    int inc = my;
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane == 31) wsum[warp] = inc;
    for (int c = 0; c < 3; ++c)
        if (myc[c]) atomicAdd(&ctot[c], myc[c]);
    __syncthreads();
    int pos = inc - my;
    for (int w = 0; w < warp; ++w) pos += wsum[w];
    for (int w = w0; w < w1; ++w) {
        unsigned m = bm[w];
        const int c = w / W, wr = w - c * W;
        while (m) {
            const int bit = __ffs(m) - 1;
            m &= m - 1;
            const int cell = order[wr * 32 + bit];
            list_cell[mbase + pos] = cell;
            list_dlt[mbase + pos] = geo[cell].dlt;
            if (c == CLS_DIRECT) {
                double t, b;
                region_cell_value(table, r0, r1, cell / grid, cell % grid, delta_grid, t_star, t_diff_spot,
                                  t_diff_fac, t, b);
                list_aux[mbase + pos] = make_double2(t, b);
            }
            ++pos;
        }
    }
    if (tid == 0) {
        int *o = counts + 4 * l;
        o[0] = ctot[0];
        o[1] = ctot[1];
        o[2] = ctot[2];
        o[3] = 0;
    }
}

// Phase lists without maps and without a cell order: one block per phase collects the
// active cells of its region boxes (as k_fir_blists) and sorts them in shared memory by
// (class, mu bin key, order-preserving image of the slope, cell index) -- a bitonic
// network over a power-of-two capacity at least the phase's box cells.  That is the
// order the two radix sorts of the cell order give (by slope, then stably by mu bin),
// so the lists are the same as k_fir_blists's, without the G*G sort.
constexpr int FIR_SLIST_THREADS = 1024;
constexpr int FIR_SLIST_CAP_MAX = 8192;

__global__ void __launch_bounds__(FIR_SLIST_THREADS)
    k_fir_slists(int grid, double delta_grid, const RegionPhase *__restrict__ table, const int *__restrict__ reg_off,
                 int t_star, int t_diff_spot, int t_diff_fac, int solar, int cap, const CellGeo *__restrict__ geo,
                 int *list_cell, double *list_dlt, double2 *list_aux, int *counts, int *status) {
    extern __shared__ __align__(16) unsigned char sl_smem[];
    // the record of an active cell in two words, compared as one 128-bit key:
    // k1 = (class << 16 | bin key) << 32 | ord64(dlt) >> 32, k2 = ord64(dlt) << 32 | cell;
    // sorted through one 64-bit word per record, sk = class and bin (12 bits) | the slope
    // image's top 32 bits | the record's index (20 bits), then each run of equal
    // (class, bin, top slope bits) is put in k2 order
    unsigned long long *k1 = reinterpret_cast<unsigned long long *>(sl_smem);   // [cap]
    unsigned long long *k2 = k1 + cap;                                         // [cap]
    unsigned long long *sk = k2 + cap;                                         // [cap]
    __shared__ int cnt, ccnt[3];
    const long long gm = (long long)grid * grid;
    const int l = blockIdx.x, tid = threadIdx.x;
    const long long mbase = (long long)l * gm;
    if (tid == 0) cnt = 0;
    if (tid < 3) ccnt[tid] = 0;
    __syncthreads();
    const int r0 = reg_off[l], r1 = reg_off[l + 1];
    const float delta_f = (float)delta_grid;
    for (int r = r0; r < r1; ++r) {
        const RegionPhase rp = table[r];
        const int by = rp.iy1 - rp.iy0, bz = rp.iz1 - rp.iz0;
        if (!rp.visible || by <= 0 || bz <= 0) continue;
        const int nbox = by * bz;
        for (int q = tid; q < nbox; q += FIR_SLIST_THREADS) {
            const int iy = rp.iy0 + q / bz, iz = rp.iz0 + q % bz;
            int owner = region_owner_fp32(table, r0, r1, iy, iz, delta_f);
            if (owner == -2) {
                double t, b;
                owner = region_cell_value(table, r0, r1, iy, iz, delta_grid, t_star, t_diff_spot, t_diff_fac, t, b);
            }
            if (owner != r) continue;
            const int k = iy * grid + iz;
            const CellGeo &g = geo[k];
            const int c = fir_class_box(g, rp.type, solar);
            if (c < 0) continue;
            atomicAdd(&ccnt[c], 1);
            const int pos = atomicAdd(&cnt, 1);
            if (pos < cap) {
                const unsigned long long od = soap_ord64(g.dlt);
                const unsigned bin = (unsigned)(g.row * 2 + g.zero_v);
                const unsigned ka = ((unsigned)c << 16) | bin;
                k1[pos] = ((unsigned long long)ka << 32) | (od >> 32);
                k2[pos] = (od << 32) | (unsigned)k;
                sk[pos] = ((unsigned long long)(((unsigned)c << 9) | bin) << 52) | ((od >> 32) << 20) |
                          (unsigned long long)pos;
            }
        }
    }
    __syncthreads();
    const int n = cnt;
    if (n > cap) {   // the host sizes cap from the boxes: cannot happen
        if (tid == 0) atomicExch(status, FIR_ST_SEGMENTS);
        if (tid < 4) counts[4 * l + tid] = 0;
        return;
    }
    int np = 1, lnp = 0;
    while (np < n) np <<= 1, ++lnp;
    for (int i = n + tid; i < np; i += FIR_SLIST_THREADS) sk[i] = ~0ULL;   // padding sorts last
    __syncthreads();
    // bitonic network over the np / 2 compare-exchange pairs of each stage: pair m of
    // stage (k, j) joins i (m with a zero bit inserted at bit log2 j) and i + j
    const int half = np >> 1;
    for (int lk = 1; lk <= lnp; ++lk) {
        for (int lj = lk - 1; lj >= 0; --lj) {
            const int j = 1 << lj;
            for (int m = tid; m < half; m += FIR_SLIST_THREADS) {
                const int i = ((m >> lj) << (lj + 1)) | (m & (j - 1));
                const int p = i + j;
                const unsigned long long a = sk[i], b = sk[p];
                if ((a > b) == (((i >> lk) & 1) == 0)) {
                    sk[i] = b;
                    sk[p] = a;
                }
            }
            __syncthreads();
        }
    }
    // runs of equal (class, bin, top slope bits): order by k2 (the slope's low bits, then
    // the cell); a run is sorted by the thread at its start (runs are short: mostly the
    // cells mirrored across the equator, whose slopes are equal)
    for (int i = tid; i < n; i += FIR_SLIST_THREADS) {
        const unsigned long long key = sk[i] >> 20;
        if (i > 0 && (sk[i - 1] >> 20) == key) continue;
        int e = i + 1;
        while (e < n && (sk[e] >> 20) == key) ++e;
        for (int a = i + 1; a < e; ++a) {   // insertion sort of [i, e) by k2
            const unsigned long long v = sk[a];
            const unsigned long long kv = k2[v & 0xfffffULL];
            int b = a - 1;
            while (b >= i && k2[sk[b] & 0xfffffULL] > kv) {
                sk[b + 1] = sk[b];
                --b;
            }
            sk[b + 1] = v;
        }
    }
    __syncthreads();
    for (int i = tid; i < n; i += FIR_SLIST_THREADS) {
        const int rec = (int)(sk[i] & 0xfffffULL);
        const int cell = (int)(unsigned)k2[rec];
        list_cell[mbase + i] = cell;
        list_dlt[mbase + i] = geo[cell].dlt;
        if ((int)(k1[rec] >> 48) == CLS_DIRECT) {
            double t, b;
            region_cell_value(table, r0, r1, cell / grid, cell % grid, delta_grid, t_star, t_diff_spot, t_diff_fac, t,
                              b);
            list_aux[mbase + i] = make_double2(t, b);
        }
    }
    if (tid == 0) {
        int *o = counts + 4 * l;
        o[0] = ccnt[0];
        o[1] = ccnt[1];
        o[2] = ccnt[2];
        o[3] = 0;
    }
}

int fir_sorted_box_capacity(long long max_box_cells) {
    int cap = 32;
    while (cap < max_box_cells) cap <<= 1;
    return cap <= FIR_SLIST_CAP_MAX ? cap : 0;
}

static size_t fir_blists_smem(long long gm) { return sizeof(unsigned) * 3 * (size_t)((gm + 31) >> 5); }

long long fir_box_lists_max_gm() { return (long long)(FIR_BLIST_SMEM_MAX / (3 * sizeof(unsigned))) * 32; }

// --- prefix sums and segments -------------------------------------------------------
template <int NV>
__device__ __forceinline__ void block_scan_excl(double (&v)[NV], int &vi, double (&tot)[NV], int &toti,
                                                double (*ws)[NV + 1]) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    double inc[NV];
    int inci = vi;
#pragma unroll
    for (int q = 0; q < NV; ++q) inc[q] = v[q];
    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double t = __shfl_up_sync(0xffffffffu, inc[q], o);
            if (lane >= o) inc[q] += t;
        }
        int ti = __shfl_up_sync(0xffffffffu, inci, o);
        if (lane >= o) inci += ti;
    }
    if (lane == 31) {
#pragma unroll
        for (int q = 0; q < NV; ++q) ws[warp][q] = inc[q];
        ws[warp][NV] = (double)inci;
    }
    __syncthreads();
    double off[NV];
    int offi = 0;
#pragma unroll
    for (int q = 0; q < NV; ++q) off[q] = 0.0, tot[q] = 0.0;
    toti = 0;
    for (int w = 0; w < nw; ++w) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            if (w < warp) off[q] += ws[w][q];
            tot[q] += ws[w][q];
        }
        int wi = (int)ws[w][NV];
        if (w < warp) offi += wi;
        toti += wi;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = off[q] + inc[q] - v[q];
    vi = offi + inci - vi;
}

// Block (l, c) for classes 0 and 1: exclusive FP64 prefix sums over the class list of
// L, L dlt, L offir and (1 + LB) L, (1 + LB) L dlt, (1 + LB) L offir (the prefix of
// the entry at list position q is stored at index q + c, the class total after its
// last entry), and the list of (mu bin, v == 0) segments:
// segs[(l*2 + c)*cap + s] = (first position, row * 2 + zero_v), nseg[l*2 + c].
__global__ void __launch_bounds__(256) k_fir_prefix(long long gm, const int *__restrict__ counts,
                                                    const int *__restrict__ list_cell,
                                                    const CellGeo *__restrict__ geo, double *pre, long long pre_stride,
                                                    long long pre_comp, int2 *segs, int *nseg, int seg_cap,
                                                    int *status) {
    const int l = blockIdx.x, c = blockIdx.y, tid = threadIdx.x;
    const int *cn = counts + 4 * l;
    const int cs = (c == 0) ? 0 : cn[0];
    const int cnt = cn[c];
    const long long lbase = (long long)l * gm;
    const long long pbase = (long long)l * pre_stride + c;
    __shared__ double ws[256 / 32][7];
    const int per = (cnt + blockDim.x - 1) / blockDim.x;
    const int a = cs + min(cnt, tid * per), b = cs + min(cnt, (tid + 1) * per);
    auto key_at = [&](int q) -> int {
        const CellGeo &g = geo[list_cell[lbase + q]];
        return g.row * 2 + g.zero_v;
    };
    double s[6] = {0, 0, 0, 0, 0, 0};
    int ns = 0;
    int prev = (a > cs && a < b) ? key_at(a - 1) : -1;
    for (int q = a; q < b; ++q) {
        const CellGeo &g = geo[list_cell[lbase + q]];
        s[0] += g.L;
        s[1] += g.L * g.dlt;
        s[2] += g.L * g.offir;
        s[3] += g.w2;
        s[4] += g.w2 * g.dlt;
        s[5] += g.w2 * g.offir;
        int k = g.row * 2 + g.zero_v;
        if (q == cs || k != prev) ns++;
        prev = k;
    }
    double tot[6];
    int tns;
    block_scan_excl<6>(s, ns, tot, tns, ws);
    prev = (a > cs && a < b) ? key_at(a - 1) : -1;
    for (int q = a; q < b; ++q) {
        const CellGeo &g = geo[list_cell[lbase + q]];
        long long pi = pbase + q;
        pre[pi] = s[0];
        pre[pre_comp + pi] = s[1];
        pre[2 * pre_comp + pi] = s[2];
        pre[3 * pre_comp + pi] = s[3];
        pre[4 * pre_comp + pi] = s[4];
        pre[5 * pre_comp + pi] = s[5];
        s[0] += g.L;
        s[1] += g.L * g.dlt;
        s[2] += g.L * g.offir;
        s[3] += g.w2;
        s[4] += g.w2 * g.dlt;
        s[5] += g.w2 * g.offir;
        int k = g.row * 2 + g.zero_v;
        if (q == cs || k != prev) {
            if (ns < seg_cap) segs[(long long)(l * 2 + c) * seg_cap + ns] = make_int2(q, k);
            ns++;
        }
        prev = k;
    }
    if (tid == 0) {
        long long pi = pbase + cs + cnt;
        for (int q = 0; q < 6; ++q) pre[q * pre_comp + pi] = tot[q];
        if (tns > seg_cap) atomicExch(status, FIR_ST_SEGMENTS);
        nseg[l * 2 + c] = min(tns, seg_cap);
    }
}

// --- device helpers of the tile kernel -------------------------------------------------
// per-pixel sums of the FP32 form: compensated (Kahan) when set
constexpr bool FIR_COMPENSATED = true;

template <typename T, bool COMP = FIR_COMPENSATED>
struct Acc {
    T s, c;
    __device__ __forceinline__ void zero() { s = (T)0; c = (T)0; }
    __device__ __forceinline__ void add(T x) {
        if constexpr (sizeof(T) == 4 && COMP) {
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

// Source position of a cell at j0 on the FP32 pipe: u0 = j0 + t with t = j0 dlt - offir
// in float pairs (exact products by fmaf, TwoSum for the sums); i0 = floor(u0),
// phi = u0 - i0.  |t| < 2^20 and j0 < 2^24.
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

// a cell's owner i0 and weight phi at j0 with its constants
template <typename T>
__device__ __forceinline__ void cell_pos(int j0, const CellGeo *geo, const CellGeo32 *geo32, int cell, int &i0,
                                         T &phi, T &dlt, T &L, T &w2) {
    if constexpr (sizeof(T) == 4) {
        CellGeo32 h = geo32[cell];
        float ph;
        fir_pos32(j0, h.a.x, h.a.y, h.a.z, h.a.w, i0, ph);
        phi = ph;
        L = h.b.x;
        w2 = h.b.y;
        dlt = h.b.z;
    } else {
        const CellGeo &g = geo[cell];
        double u0 = fma((double)j0, g.ir, -g.offir);
        double fl = floor(u0);
        i0 = (int)fl;
        phi = u0 - fl;
        L = g.L;
        w2 = g.w2;
        dlt = g.dlt;
    }
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

// mbarrier + bulk copy (TMA, non-tensor form)
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity,
                                                  long long limit = FIR_WAIT_LIMIT) {
    for (long long it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

struct FirCubes {
    // PHASE: c[0] the spot class's rows per pixel (q_sed, q_norm, spot_norm, q_norm -
    // spot_norm), c[1] the facula class's (q_sed, q_norm - fac_norm, q_norm, fac_norm),
    // each n_mu x n Vec4 -- the order in which a unit's four sums use them; QUIET: c[0],
    // one cube of T.  Workspace slots: 256-byte aligned, padded to 256 bytes.
    const void *c[6];
    const double *spot_sed;
    const double *fac_sed;
    // FP32 form: the two continuum rows as float pairs (hi, lo)
    const float2 *spot_sed2;
    const float2 *fac_sed2;
};

// cube rows staged for a segment of class cls (window slot q)
//   spot:   S (q_sed), Qs (q_norm), As (spot_norm), Bs (q_norm - spot_norm)  -- weight L
//   facula: S (q_sed), Bf (q_norm - fac_norm) -- weight L; Qf (q_norm), Af (fac_norm) -- weight (1+LB) L
__device__ __forceinline__ int fir_cube_index(int mode, int cls, int q) {
    if (mode == MODE_QUIET) return 0;
    if (cls == CLS_SPOT) return q;
    return (q == 0) ? 0 : (q == 1) ? 5 : (q == 2) ? 1 : 4;
}

struct FirSeg {
    int start, end;     // list positions
    int key;            // row * 2 + zero_v
    int cls;
    int m_lo, m_hi;     // floor of t over the segment and the tile
    int u0;             // first work unit
};

// one work unit: a segment's shift values [ma, mb] with the source window they read
struct FirUnit {
    int cls, key;       // class, row * 2 + zero_v
    int start, end;     // the segment's list positions
    int m_lo, m_hi;     // the segment's shift range at this tile
    int ma, mb;         // this unit's shift values
    int w0, w1, off;    // window [w0, w1) (source pixels), offset of w0 in the staged copy
};

template <typename T>
struct FirGrp {
    T a0, a1, b;        // weight L
    T a0w, a1w, bw;     // weight (1 + LB) L (faculae)
    int m, ok;
};

template <typename T>
struct FirExcW {        // wrap cell of a unit (reads the staged window)
    int i0;
    T phi, dlt, L, w2;
};

template <typename T>
struct FirExcD {        // directly evaluated cell (reads the cubes in global memory)
    int i0, row, kind, zero_v;
    T phi, dlt, L, w2;
    double temp;
};

// Plan of (a batch of) a tile's work units: units, one group per shift value (task),
// and the wrap cells.  U units, G tasks, E wrap cells at most.
template <typename T, int U, int G, int E>
struct FirPlanSt {
    static constexpr int NU = U, NG = G, NE = E;
    FirUnit unit[U];
    int ut[U + 1];          // first task of each unit; ut[nb] = ntask
    FirGrp<T> grp[G];
    int wlo[G];             // first list position of each task's wrap cells
    int woff[G + 1];        // exclusive offsets of the tasks' wrap cells; woff[ntask] = etot
    FirExcW<T> excw[E];
    int nunit, nb, ntask, etot, ok;
};

// the tile kernel's batches, and the plans precomputed per tile by k_fir_plan
template <typename T>
using FirTileSt = FirPlanSt<T, 128, (sizeof(T) == 4) ? 512 : 256, (sizeof(T) == 4) ? 512 : 256>;
template <typename T>
using FirPrePlan = FirPlanSt<T, 32, 128, 128>;
// one warp per (list, tile): the plan's block barriers are then a single warp's
// (0.106 ms per 100-phase step against 0.112 with 64 threads and 0.152 with 128)
constexpr int FIR_PLAN_THREADS = 32;

// Compact plan record of one (list, tile) as the plan kernel writes it: int4 header
// (units, tasks, wrap cells, ok) at 0, then units, ut[nb + 1], woff[ntask + 1], groups and
// wrap cells, each 8-byte aligned; records sit in slots of FirPlanSlot<T>::BYTES and are
// copied whole (bytes = the record's size, a multiple of 16) into shared memory.
template <typename T>
struct FirPlanLayout {
    int o_unit, o_ut, o_woff, o_grp, o_exc, bytes;
    __host__ __device__ constexpr FirPlanLayout(int nb, int ntask, int etot)
        : o_unit(16),
          o_ut((16 + (int)sizeof(FirUnit) * nb + 7) & ~7),
          o_woff((((16 + (int)sizeof(FirUnit) * nb + 7) & ~7) + 4 * (nb + 1) + 7) & ~7),
          o_grp((((((16 + (int)sizeof(FirUnit) * nb + 7) & ~7) + 4 * (nb + 1) + 7) & ~7) + 4 * (ntask + 1) + 7) & ~7),
          o_exc(0),
          bytes(0) {
        o_exc = (o_grp + (int)sizeof(FirGrp<T>) * ntask + 7) & ~7;
        bytes = (o_exc + (int)sizeof(FirExcW<T>) * etot + 15) & ~15;
    }
};
template <typename T>
struct FirPlanSlot {
    static constexpr int BYTES = FirPlanLayout<T>(FirPrePlan<T>::NU, FirPrePlan<T>::NG, FirPrePlan<T>::NE).bytes;
};

// lists of at most this many (class 0 + 1) entries have their slopes staged in shared
// memory for the tile kernel's own searches
template <typename T>
struct FirListCap {
    static constexpr int N = (sizeof(T) == 4) ? 4096 : 1024;
};

template <typename T, int NC>
struct FirSmem {
    // staged windows; the direct cells' buffer reuses this space once all copies landed
    union {
        T win[2][NC][FIR_WIN];
        FirExcD<T> excd[FIR_EXC];
    };
    unsigned long long bar[2];
    FirTileSt<T> st;
    int wsum[FIR_THREADS / 32];
    int fail;
    double sdl[FirListCap<T>::N];          // the list's slopes (short lists)
    // followed by FirSeg seg[] (dynamic, 16-byte aligned)
};

template <typename T, int NC>
__host__ __device__ constexpr size_t fir_smem_fixed() { return (sizeof(FirSmem<T, NC>) + 15) & ~size_t(15); }

template <int NT>
__device__ __forceinline__ int block_excl_scan_int(int v, int *wsum, int &total) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    int off = 0, tot = 0;
    for (int w = 0; w < NT / 32; ++w) {
        if (w < warp) off += wsum[w];
        tot += wsum[w];
    }
    __syncthreads();
    total = tot;
    return off + inc - v;
}

// First position q in [lo, hi) with dlt_q >= theta_m, theta_m = m (1 / X) rounded: the
// cells whose t = dlt X reaches m.  theta_m is monotone in m and the slopes ascend, so
// the ranges of consecutive m partition the segment exactly; the comparisons run on the
// order-preserving integer images of the doubles (no FP64 instruction per step).  A cell
// within rounding of a boundary may be classified one group away from floor(t); its
// weight is then within rounding of 0 or 1 and its contribution unchanged.
// Four lower-bound searches over the same range [lo, hi) of a list's slopes (sorted):
// out[q] = the first position whose slope's ord64 image is >= th[q] (th[q] = the image
// of m / X for a boundary shift m and a pixel position X).  In lock-step, so the four
// loads of a step are in flight together; each search halves its own interval.
__device__ __forceinline__ void fir_lower_bound4(const double *__restrict__ dl, int lo, int hi,
                                                 const unsigned long long (&th)[4], int (&out)[4]) {
    int l[4] = {lo, lo, lo, lo}, h[4] = {hi, hi, hi, hi};
    while (l[0] < h[0] || l[1] < h[1] || l[2] < h[2] || l[3] < h[3]) {
        unsigned long long v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = (l[q] < h[q]) ? soap_ord64(dl[(l[q] + h[q]) >> 1]) : 0ULL;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (l[q] < h[q]) {
                const int mid = (l[q] + h[q]) >> 1;
                if (v[q] >= th[q]) h[q] = mid;
                else l[q] = mid + 1;
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) out[q] = l[q];
}

struct FirTileArgs {
    int n, n_eff;
    const double *lam;
    double los;                 // lambda0 / step
    FirCubes cubes;
    const int *list_cell;       // [l][gm]
    const double *list_dlt;     // [l][gm]
    const int *counts;          // [l][4]
    const double *pre;          // 6 components x [l][pre_stride]
    long long pre_stride, pre_comp;
    const int2 *segs;           // [l][2][seg_cap]
    const int *nseg;            // [l][2]
    int seg_cap;
    const CellGeo *geo;
    const CellGeo32 *geo32;
    const double2 *list_aux;    // [l][gm]: (temperature, type) of the directly evaluated entries
    long long gm;
    int solar, t_norm_fac;
    void *out0, *out1, *out2;
    long long out_stride;
    int *status;
    const void *plan;           // FirPrePlan<T> per (list, tile), or null
    const int *run_list;        // lists to integrate (ascending), or null for all of them
    int n_lists_all;            // lists with a plan slot
    long long wait_limit;       // polls per bounded wait of the persistent kernel
    int drop_plan;              // failure-path test: the first plan copy is expected, not issued
    int drop_unit;              // failure-path test: each block's first window copy is expected, not issued
};

// The list's (class, mu bin, v == 0) segments with their shift ranges at the tile
// [j0, j0 + t_eff) and first work units; returns the number of units.  Block-wide.
template <int MODE, int NT>
__device__ int fir_segments(const FirTileArgs &A, int l, int j0, int t_eff, FirSeg *segs, int nsg, int *nunit_sh) {
    const int tid = threadIdx.x;
    const double *dl = A.list_dlt + (long long)l * A.gm;
    const int *cn = A.counts + 4 * l;
    const int ns0 = A.nseg[2 * l];
    const int ns1 = nsg - ns0;
    const double Xa = (double)j0 + A.los, Xb = (double)(j0 + t_eff - 1) + A.los;
    for (int s = tid; s < nsg; s += NT) {
        const int c = (s < ns0) ? 0 : 1;
        const int si = (c == 0) ? s : s - ns0;
        const int ns_c = (c == 0) ? ns0 : ns1;
        const int2 *sp = A.segs + (long long)(2 * l + c) * A.seg_cap;
        const int2 e = sp[si];
        const int cend = (c == 0) ? cn[0] : cn[0] + cn[1];
        FirSeg g;
        g.start = e.x;
        g.end = (si + 1 < ns_c) ? sp[si + 1].x : cend;
        g.key = e.y;
        g.cls = c;
        const double d0 = dl[g.start], d1 = dl[g.end - 1];
        // one more shift value on either side covers the cells the searches' thresholds
        // classify one group away from floor(t)
        g.m_lo = (int)fmin(floor(d0 * Xa), floor(d0 * Xb)) - 1;
        g.m_hi = (int)fmax(floor(d1 * Xa), floor(d1 * Xb)) + 1;
        if (fmax(fabs(d0), fabs(d1)) * (double)(FIR_TILE - 1) >= 1.0) {
            atomicExch(A.status, FIR_ST_FAST);   // a weight could wrap twice in one tile
            g.m_hi = g.m_lo;
        }
        g.u0 = 0;
        segs[s] = g;
    }
    __syncthreads();
    if (tid == 0) {   // work units: ceil((m_hi - m_lo + 1) / FIR_MCH) per segment
        int u = 0;
        for (int s = 0; s < nsg; ++s) {
            segs[s].u0 = u;
            u += (segs[s].m_hi - segs[s].m_lo + FIR_MCH) / FIR_MCH;
        }
        *nunit_sh = u;
    }
    __syncthreads();
    return *nunit_sh;
}

// descriptor of work unit u: its segment, shift values and source window
// (PHASE: the staged rows are Vec4 elements, 16-byte aligned, so the window starts at
// its first pixel; QUIET: rows of T, staged from the 16-byte boundary below w0)
template <typename T, int MODE>
__device__ __forceinline__ FirUnit fir_describe(int u, const FirSeg *segs, int nsg, int j0, int t_eff, int n,
                                                int n_eff) {
    int lo = 0, hi = nsg - 1;
    while (lo < hi) {   // last segment with u0 <= u
        int mid = (lo + hi + 1) >> 1;
        if (segs[mid].u0 <= u) lo = mid; else hi = mid - 1;
    }
    const FirSeg &g = segs[lo];
    FirUnit d;
    d.cls = g.cls;
    d.key = g.key;
    d.start = g.start;
    d.end = g.end;
    d.m_lo = g.m_lo;
    d.m_hi = g.m_hi;
    d.ma = g.m_lo + (u - g.u0) * FIR_MCH;
    d.mb = min(g.m_hi, d.ma + FIR_MCH - 1);
    d.w0 = max(0, j0 + d.ma - (d.ma > g.m_lo ? 1 : 0));
    d.w1 = min(n_eff, j0 + t_eff + d.mb + 1);
    d.off = (MODE == MODE_PHASE || d.w1 <= d.w0)
                ? 0
                : (int)(((((long long)(g.key >> 1) * n + d.w0) * (long long)sizeof(T)) & 15) / (long long)sizeof(T));
    return d;
}

// wrap cells [lo, hi) of a plan into st.excw[e - dst0]
template <typename T, int NT, typename ST>
__device__ __forceinline__ void fir_fill_exc(const FirTileArgs &A, int l, int j0, ST &st, int lo, int hi, int dst0) {
    const long long lbase = (long long)l * A.gm;
    for (int e = lo + (int)threadIdx.x; e < hi; e += NT) {
        int a = 0, b = st.ntask - 1;
        while (a < b) {   // last task with woff <= e
            int mid = (a + b + 1) >> 1;
            if (st.woff[mid] <= e) a = mid; else b = mid - 1;
        }
        const int cell = A.list_cell[lbase + st.wlo[a] + (e - st.woff[a])];
        FirExcW<T> x;
        cell_pos<T>(j0, A.geo, A.geo32, cell, x.i0, x.phi, x.dlt, x.L, x.w2);
        st.excw[e - dst0] = x;
    }
}

// Plan of the units [ub, ub + nb): as many as fit ST's capacities, their groups (binary
// searches on the slopes sl, coefficients from the prefix sums) and wrap ranges, and
// the first ST::NE wrap cells.  Block-wide; sets st.nb, st.ntask, st.etot.
template <typename T, int MODE, int NT, typename ST>
__device__ void fir_plan_batch(const FirTileArgs &A, int l, int j0, int t_eff, const FirSeg *segs, int nsg,
                               int nunit, const double *sl, ST &st, int ub, int *wsum) {
    const int tid = threadIdx.x;
    const int n = A.n, n_eff = A.n_eff;
    const double dj0 = soap_i2d(j0);
    const double iXa = 1.0 / (dj0 + A.los), iXb = 1.0 / (soap_i2d(j0 + t_eff - 1) + A.los);
    const int nbu = min(ST::NU, nunit - ub);
    for (int t = tid; t < nbu; t += NT) st.unit[t] = fir_describe<T, MODE>(ub + t, segs, nsg, j0, t_eff, n, n_eff);
    __syncthreads();
    if (tid == 0) {
        int nb = 0, nt = 0;
        st.ut[0] = 0;
        while (nb < nbu) {
            const int k = st.unit[nb].mb - st.unit[nb].ma + 1;
            if (nt + k > ST::NG) break;
            nt += k;
            st.ut[++nb] = nt;
        }
        st.nb = nb;
        st.ntask = nt;
    }
    __syncthreads();
    const int nb = st.nb, ntask = st.ntask;
    for (int k = tid; k < ntask; k += NT) {
        int ui = 0, hi = nb - 1;
        while (ui < hi) {   // unit of task k
            int mid = (ui + hi + 1) >> 1;
            if (st.ut[mid] <= k) ui = mid; else hi = mid - 1;
        }
        const FirUnit d = st.unit[ui];
        const int m = d.ma + (k - st.ut[ui]);
        const double dm = soap_i2d(m), dm1 = soap_i2d(m + 1);
        // the four boundaries in lock-step (those at the unit's first and last shift are
        // the range's ends)
        const unsigned long long th[4] = {soap_ord64(dm * iXa), soap_ord64(dm * iXb), soap_ord64(dm1 * iXa),
                                          soap_ord64(dm1 * iXb)};
        int bnd[4];
        fir_lower_bound4(sl, d.start, d.end, th, bnd);
        const int lowA = (m == d.m_lo) ? d.start : bnd[0], lowB = (m == d.m_lo) ? d.start : bnd[1];
        const int highA = (m == d.m_hi) ? d.end : bnd[2], highB = (m == d.m_hi) ? d.end : bnd[3];
        const int rlo = max(lowA, lowB), rhi = min(highA, highB);
        FirGrp<T> gr;
        gr.m = m;
        gr.ok = rhi > rlo;
        gr.a0 = gr.a1 = gr.b = gr.a0w = gr.a1w = gr.bw = (T)0;
        if (gr.ok) {
            const double *P = A.pre + (long long)l * A.pre_stride + d.cls;
            const long long pc = A.pre_comp;
            const double SL = P[rhi] - P[rlo];
            const double SLd = P[pc + rhi] - P[pc + rlo];
            const double SLo = P[2 * pc + rhi] - P[2 * pc + rlo];
            const double A1 = dj0 * SLd - SLo - dm * SL;
            gr.a1 = soap_to<T>(A1);
            gr.a0 = soap_to<T>(SL - A1);
            gr.b = soap_to<T>(SLd);
            if (MODE == MODE_PHASE && d.cls == CLS_FAC) {
                const double Wt = P[3 * pc + rhi] - P[3 * pc + rlo];
                const double Wd = P[4 * pc + rhi] - P[4 * pc + rlo];
                const double Wo = P[5 * pc + rhi] - P[5 * pc + rlo];
                const double W1 = dj0 * Wd - Wo - dm * Wt;
                gr.a1w = soap_to<T>(W1);
                gr.a0w = soap_to<T>(Wt - W1);
                gr.bw = soap_to<T>(Wd);
            }
        }
        st.grp[k] = gr;
        int wl = 0, wc = 0;
        if (m > d.m_lo) {   // cells whose floor changes across boundary m inside the tile
            wl = min(lowA, lowB);
            wc = max(lowA, lowB) - wl;
        }
        st.wlo[k] = wl;
        st.woff[k] = wc;
    }
    __syncthreads();
    {   // exclusive offsets of the wrap counts (NG / NT entries per thread)
        constexpr int PER = ST::NG / NT;
        static_assert(ST::NG % NT == 0, "task capacity per thread");
        const int a = tid * PER;
        int loc = 0;
#pragma unroll
        for (int q = 0; q < PER; ++q)
            if (a + q < ntask) loc += st.woff[a + q];
        int etot;
        int ex = block_excl_scan_int<NT>(loc, wsum, etot);
#pragma unroll
        for (int q = 0; q < PER; ++q)
            if (a + q < ntask) {
                int v = st.woff[a + q];
                st.woff[a + q] = ex;
                ex += v;
            }
        if (tid == 0) {
            st.woff[ntask] = etot;
            st.etot = etot;
        }
    }
    __syncthreads();
    fir_fill_exc<T, NT>(A, l, j0, st, 0, min(st.etot, ST::NE), 0);
    __syncthreads();
}

// Plans of every (list, tile) of the phase integration, computed ahead of the tile
// kernel by small blocks (many per SM, so that the searches' load latencies overlap
// across tiles).  A tile whose units, groups or wrap cells exceed FirPrePlan's
// capacities gets ok = 0 and plans itself in the tile kernel.
template <typename T>
__global__ void __launch_bounds__(FIR_PLAN_THREADS) k_fir_plan(const FirTileArgs A) {
    extern __shared__ __align__(16) unsigned char plan_smem[];
    FirPrePlan<T> &st = *reinterpret_cast<FirPrePlan<T> *>(plan_smem);
    __shared__ int wsum[FIR_PLAN_THREADS / 32];
    __shared__ int nunit_sh;
    FirSeg *segs = reinterpret_cast<FirSeg *>(plan_smem + ((sizeof(FirPrePlan<T>) + 15) & ~size_t(15)));
    const int l = A.run_list ? A.run_list[blockIdx.y] : (int)blockIdx.y;
    const int j0 = blockIdx.x * FIR_TILE, tid = threadIdx.x;
    const long long tau = (long long)l * gridDim.x + blockIdx.x;
    const long long ntot = (long long)gridDim.x * A.n_lists_all;
    char *rec = reinterpret_cast<char *>(const_cast<void *>(A.plan)) + tau * FirPlanSlot<T>::BYTES;
    int *psize = reinterpret_cast<int *>(reinterpret_cast<char *>(const_cast<void *>(A.plan)) +
                                         ntot * FirPlanSlot<T>::BYTES);
    const int t_eff = min(FIR_TILE, A.n_eff - j0);
    if (t_eff <= 0) {
        if (tid == 0) {
            *reinterpret_cast<int4 *>(rec) = make_int4(0, 0, 0, 1);
            psize[tau] = 16;
        }
        return;
    }
    const int nsg = A.nseg[2 * l] + A.nseg[2 * l + 1];
    const int nunit = fir_segments<MODE_PHASE, FIR_PLAN_THREADS>(A, l, j0, t_eff, segs, nsg, &nunit_sh);
    int ok = 1;
    if (nunit > FirPrePlan<T>::NU) {
        ok = 0;
    } else if (nunit > 0) {
        fir_plan_batch<T, MODE_PHASE, FIR_PLAN_THREADS>(A, l, j0, t_eff, segs, nsg, nunit,
                                                        A.list_dlt + (long long)l * A.gm, st, 0, wsum);
        ok = (st.nb == nunit) && (st.etot <= FirPrePlan<T>::NE);
    } else if (tid == 0) {
        st.nb = st.ntask = st.etot = 0;
        st.ut[0] = 0;
        st.woff[0] = 0;
    }
    __syncthreads();
    const int nb = ok ? st.nb : 0, ntask = ok ? st.ntask : 0, etot = ok ? st.etot : 0;
    const FirPlanLayout<T> L(nb, ntask, etot);
    if (ok) {   // the used parts, compact
        FirUnit *u = reinterpret_cast<FirUnit *>(rec + L.o_unit);
        int *ut = reinterpret_cast<int *>(rec + L.o_ut);
        int *wo = reinterpret_cast<int *>(rec + L.o_woff);
        FirGrp<T> *gr = reinterpret_cast<FirGrp<T> *>(rec + L.o_grp);
        FirExcW<T> *ex = reinterpret_cast<FirExcW<T> *>(rec + L.o_exc);
        for (int i = tid; i < nb; i += FIR_PLAN_THREADS) u[i] = st.unit[i];
        for (int i = tid; i <= nb; i += FIR_PLAN_THREADS) ut[i] = st.ut[i];
        for (int i = tid; i <= ntask; i += FIR_PLAN_THREADS) wo[i] = st.woff[i];
        for (int i = tid; i < ntask; i += FIR_PLAN_THREADS) gr[i] = st.grp[i];
        for (int i = tid; i < etot; i += FIR_PLAN_THREADS) ex[i] = st.excw[i];
    }
    if (tid == 0) {
        *reinterpret_cast<int4 *>(rec) = make_int4(nb, ntask, etot, ok);
        psize[tau] = ok ? L.bytes : 16;
    }
}

// QUIET: OutT = double (one spectrum, once per star); PHASE: OutT = T (the FP32 form
// keeps its deficits in FP32 for the FP32 convolution that consumes them)
template <typename T, int MODE, typename OutT>
__global__ void __launch_bounds__(FIR_THREADS) k_fir(const FirTileArgs A) {
    constexpr int NC = (MODE == MODE_QUIET) ? 1 : 4;
    extern __shared__ __align__(128) unsigned char fir_smem[];
    FirSmem<T, NC> &sh = *reinterpret_cast<FirSmem<T, NC> *>(fir_smem);
    FirSeg *segs = reinterpret_cast<FirSeg *>(fir_smem + fir_smem_fixed<T, NC>());
    FirTileSt<T> &st = sh.st;
    const int l = blockIdx.y;
    const int j0 = blockIdx.x * FIR_TILE;
    const int tid = threadIdx.x;
    const int n = A.n, n_eff = A.n_eff;
    OutT *out0 = reinterpret_cast<OutT *>(A.out0);
    OutT *out1 = reinterpret_cast<OutT *>(A.out1);
    OutT *out2 = reinterpret_cast<OutT *>(A.out2);
    const int t_eff = min(FIR_TILE, n_eff - j0);
    if (t_eff <= 0) {   // whole tile in the zero tail [n_eff, n)
        for (int q = 0; q < FIR_PIX; ++q) {
            int j = j0 + tid + q * FIR_THREADS;
            if (j >= n) continue;
            long long o = (long long)l * A.out_stride + j;
            out0[o] = (OutT)0;
            if constexpr (MODE == MODE_PHASE) { out1[o] = (OutT)0; out2[o] = (OutT)0; }
        }
        return;
    }
    const long long lbase = (long long)l * A.gm;
    const int *cn = A.counts + 4 * l;
    if (tid == 0) {
        mbar_init(&sh.bar[0], 1);
        mbar_init(&sh.bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sh.fail = 0;
    }

    // accumulators: QUIET [0]; PHASE: S, Qs, As, Bs, Qf, Af, Bf
    constexpr int NACC = (MODE == MODE_QUIET) ? 1 : 7;
    Acc<T> acc[NACC][FIR_PIX];
#pragma unroll
    for (int a = 0; a < NACC; ++a)
#pragma unroll
        for (int q = 0; q < FIR_PIX; ++q) acc[a][q].zero();

    constexpr int EXC = FirTileSt<T>::NE;
    // staging of unit u's rows into buffer u & 1 (thread 0)
    auto issue = [&](int u, const FirUnit &d) {
        const int b = u & 1;
        unsigned bytes = 0;
        uintptr_t rel = 0;   // 16-byte aligned start, relative to the cube base
        if (d.w1 > d.w0) {
            const uintptr_t p0 = (uintptr_t)((long long)(d.key >> 1) * n + d.w0) * sizeof(T);
            const uintptr_t p1 = (uintptr_t)((long long)(d.key >> 1) * n + d.w1) * sizeof(T);
            rel = p0 & ~uintptr_t(15);
            bytes = (unsigned)(((p1 + 15) & ~uintptr_t(15)) - rel);
        }
        // the buffer was last read through the generic proxy; order those reads before
        // the async-proxy writes
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&sh.bar[b], bytes * NC);
        if (bytes) {
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                const char *base = reinterpret_cast<const char *>(A.cubes.c[fir_cube_index(MODE, d.cls, q)]);
                bulk_g2s(&sh.win[b][q][0], base + rel, bytes, &sh.bar[b]);
            }
        }
    };

    int u_fail = -1;
    int issued = -1;   // last unit whose copy was issued (thread 0)
    // apply the planned units st.unit[0, nb) (global unit numbers ub + ui)
    auto run_units = [&](int ub) {
        const int nb = st.nb, ntask = st.ntask;
        if (tid == 0 && nb > 0 && issued < ub) {
            issue(ub, st.unit[0]);
            issued = ub;
        }
        for (int ui = 0; ui < nb; ++ui) {
            const int u = ub + ui;
            if (tid == 0 && ui + 1 < nb) {
                issue(u + 1, st.unit[ui + 1]);
                issued = u + 1;
            }
            const FirUnit d = st.unit[ui];
            const int cls = d.cls, zv = d.key & 1;
            if (!mbar_wait_bounded(&sh.bar[u & 1], (unsigned)((u >> 1) & 1))) atomicExch(&sh.fail, 1);
            __syncthreads();
            if (sh.fail) {
                u_fail = u;
                return;
            }
            const T(*W)[FIR_WIN] = sh.win[u & 1];
            const int wo = d.off - d.w0;   // staged index of source pixel i: i + wo
            const int t_lo = st.ut[ui], t_hi = st.ut[ui + 1];
            for (int t = t_lo; t < t_hi; ++t) {
                const FirGrp<T> gr = st.grp[t];
                if (!gr.ok) continue;
                const int m = gr.m;
                // pixels whose owner j + m lies in [0, n_eff - 2] (v == 0: [0, n_eff - 1])
                const int jlo = max(j0, -m);
                const int jhi = zv ? j0 + t_eff - 1 : min(j0 + t_eff - 1, n_eff - 2 - m);
                // the group at the thread's pixels; CHECKED: some pixels of the tile fall
                // outside [jlo, jhi], else none and no test is needed (same arithmetic)
                auto group_at = [&](auto checked_c) {
                    constexpr bool CHECKED = decltype(checked_c)::value;
#pragma unroll
                    for (int q = 0; q < FIR_PIX; ++q) {
                        const int dj = tid + q * FIR_THREADS;
                        const int j = j0 + dj;
                        if (CHECKED && (j < jlo || j > jhi)) continue;
                        const int x = j + m + wo;
                        if (zv) {   // single tap: w == 0
                            if constexpr (MODE == MODE_QUIET) {
                                acc[0][q].add(gr.a0 * W[0][x]);
                            } else if (cls == CLS_SPOT) {
                                acc[0][q].add(gr.a0 * W[0][x]);
                                acc[1][q].add(gr.a0 * W[1][x]);
                                acc[2][q].add(gr.a0 * W[2][x]);
                                acc[3][q].add(gr.a0 * W[3][x]);
                            } else {
                                acc[0][q].add(gr.a0 * W[0][x]);
                                acc[6][q].add(gr.a0 * W[1][x]);
                                acc[4][q].add(gr.a0w * W[2][x]);
                                acc[5][q].add(gr.a0w * W[3][x]);
                            }
                            continue;
                        }
                        const T fdj = (T)dj;
                        const T c0 = gr.a0 - gr.b * fdj, c1 = gr.a1 + gr.b * fdj;
                        if constexpr (MODE == MODE_QUIET) {
                            acc[0][q].add(c0 * W[0][x] + c1 * W[0][x + 1]);
                        } else if (cls == CLS_SPOT) {
                            acc[0][q].add(c0 * W[0][x] + c1 * W[0][x + 1]);
                            acc[1][q].add(c0 * W[1][x] + c1 * W[1][x + 1]);
                            acc[2][q].add(c0 * W[2][x] + c1 * W[2][x + 1]);
                            acc[3][q].add(c0 * W[3][x] + c1 * W[3][x + 1]);
                        } else {
                            const T e0 = gr.a0w - gr.bw * fdj, e1 = gr.a1w + gr.bw * fdj;
                            acc[0][q].add(c0 * W[0][x] + c1 * W[0][x + 1]);
                            acc[6][q].add(c0 * W[1][x] + c1 * W[1][x + 1]);
                            acc[4][q].add(e0 * W[2][x] + e1 * W[2][x + 1]);
                            acc[5][q].add(e0 * W[3][x] + e1 * W[3][x + 1]);
                        }
                    }
                };
                if (jlo <= j0 && jhi >= j0 + FIR_TILE - 1) group_at(std::integral_constant<bool, false>());
                else group_at(std::integral_constant<bool, true>());
            }
            // --- wrap cells of the unit (per-cell lerp from the staged rows) ------------
            const int e_lo = st.woff[t_lo], e_hi = st.woff[t_hi];
            for (int cb = e_lo; cb < e_hi; cb += EXC) {
                const int ce = min(e_hi, cb + EXC);
                int x0 = cb;   // excw index of entry cb
                if (e_hi > EXC) {   // not all staged: refill this chunk
                    __syncthreads();
                    fir_fill_exc<T, FIR_THREADS>(A, l, j0, st, cb, ce, cb);
                    __syncthreads();
                    x0 = 0;
                }
                for (int e = cb; e < ce; ++e) {
                    const FirExcW<T> xc = st.excw[x0 + (e - cb)];
#pragma unroll
                    for (int q = 0; q < FIR_PIX; ++q) {
                        const int dj = tid + q * FIR_THREADS;
                        const int j = j0 + dj;
                        if (j >= n_eff) continue;
                        T wd = xc.phi + xc.dlt * (T)dj;
                        int i = xc.i0 + dj;
                        if (wd >= (T)1) { wd -= (T)1; i += 1; }
                        else if (wd < (T)0) { wd += (T)1; i -= 1; }
                        if (i < 0 || i > n_eff - 2) continue;
                        const int x = i + wo;
                        // the per-cell owner can differ by one from the segment's
                        // classification when t lies within rounding of an integer: such
                        // pixels read the row in global memory instead of the window
                        const bool staged = (i >= d.w0) && (i + 1 < d.w1);
                        auto lv = [&](int c) -> T {
                            T s0, s1;
                            if (staged) {
                                s0 = W[c][x];
                                s1 = W[c][x + 1];
                            } else {
                                const T *rowp = reinterpret_cast<const T *>(A.cubes.c[fir_cube_index(MODE, cls, c)]) +
                                                (long long)(d.key >> 1) * n;
                                s0 = rowp[i];
                                s1 = rowp[i + 1];
                            }
                            return s0 + (s1 - s0) * wd;
                        };
                        if constexpr (MODE == MODE_QUIET) {
                            acc[0][q].add(xc.L * lv(0));
                        } else if (cls == CLS_SPOT) {
                            acc[0][q].add(xc.L * lv(0));
                            acc[1][q].add(xc.L * lv(1));
                            acc[2][q].add(xc.L * lv(2));
                            acc[3][q].add(xc.L * lv(3));
                        } else {
                            acc[0][q].add(xc.L * lv(0));
                            acc[6][q].add(xc.L * lv(1));
                            acc[4][q].add(xc.w2 * lv(2));
                            acc[5][q].add(xc.w2 * lv(3));
                        }
                    }
                }
            }
            __syncthreads();   // unit's buffer free
        }
    };

    {
        // --- plan the tile here, batch by batch ------------------------------------------
        const int nsg = A.nseg[2 * l] + ((MODE == MODE_PHASE) ? A.nseg[2 * l + 1] : 0);
        const int nunit = fir_segments<MODE, FIR_THREADS>(A, l, j0, t_eff, segs, nsg, &st.nunit);
        // slopes of a short list in shared memory: the searches then cost no global latency
        const int n01 = cn[0] + ((MODE == MODE_PHASE) ? cn[1] : 0);
        const double *sl = A.list_dlt + lbase;
        if (n01 <= FirListCap<T>::N) {
            for (int q = tid; q < n01; q += FIR_THREADS) sh.sdl[q] = sl[q];
            sl = sh.sdl;
            __syncthreads();
        }
        for (int ub = 0; ub < nunit;) {
            fir_plan_batch<T, MODE, FIR_THREADS>(A, l, j0, t_eff, segs, nsg, nunit, sl, st, ub, sh.wsum);
            run_units(ub);
            if (u_fail >= 0) break;
            ub += st.nb;
        }
    }
    if (u_fail >= 0) {
        // a copy did not land in time: record it, give the copies still in flight (units
        // u_fail and u_fail + 1) a bounded wait, and leave without writing
        if (tid == 0) {
            atomicExch(A.status, FIR_ST_WAIT);
            mbar_wait_bounded(&sh.bar[u_fail & 1], (unsigned)((u_fail >> 1) & 1));
            if (issued > u_fail)
                mbar_wait_bounded(&sh.bar[(u_fail + 1) & 1], (unsigned)(((u_fail + 1) >> 1) & 1));
        }
        return;
    }

    // --- directly evaluated cells (class 2: spots of non-integral temperature, solar faculae)
    if constexpr (MODE == MODE_PHASE) {
        const int c_start = cn[0] + cn[1], c_cnt = cn[2];
        for (int b0 = 0; b0 < c_cnt; b0 += FIR_EXC) {
            const int nb = min(FIR_EXC, c_cnt - b0);
            if (tid < nb) {
                const int cell = A.list_cell[lbase + c_start + b0 + tid];
                FirExcD<T> x;
                cell_pos<T>(j0, A.geo, A.geo32, cell, x.i0, x.phi, x.dlt, x.L, x.w2);
                const CellGeo &gg = A.geo[cell];
                x.row = gg.row;
                x.zero_v = gg.zero_v;
                const double2 ax = A.list_aux[lbase + c_start + b0 + tid];
                x.temp = ax.x;
                x.kind = bits_is_zero(ax.y) ? 0 : 1;
                sh.excd[tid] = x;
            }
            __syncthreads();
            for (int e = 0; e < nb; ++e) {
                const FirExcD<T> xc = sh.excd[e];
                const long long off = (long long)xc.row * n;
#pragma unroll
                for (int q = 0; q < FIR_PIX; ++q) {
                    const int dj = tid + q * FIR_THREADS;
                    const int j = j0 + dj;
                    if (j >= n_eff) continue;
                    long long i;
                    T w;
                    if (xc.zero_v) {
                        i = j;
                        w = (T)0;
                    } else {
                        T wd = xc.phi + xc.dlt * (T)dj;
                        i = (long long)xc.i0 + dj;
                        if (wd >= (T)1) { wd -= (T)1; i += 1; }
                        else if (wd < (T)0) { wd += (T)1; i -= 1; }
                        if (i < 0 || i > n_eff - 2) continue;
                        w = wd;
                    }
                    auto val = [&](int ci) -> T {
                        const T *rowp = reinterpret_cast<const T *>(A.cubes.c[ci]) + off;
                        if (xc.zero_v) return rowp[i];
                        return rowp[i] + (rowp[i + 1] - rowp[i]) * w;
                    };
                    const T L = xc.L;
                    acc[0][q].add(L * val(0));                 // S (q_sed)
                    if (xc.kind == 0) {                        // spot of non-integral temperature
                        T Lq = (T)((double)L * fir_planck_ratio(A.lam[j], xc.temp, (double)(int)xc.temp));
                        acc[1][q].add(Lq * val(1));            // Qs (q_norm)
                        acc[2][q].add(Lq * val(2));            // As (spot_norm)
                        acc[3][q].add(L * val(3));             // Bs (q_norm - spot_norm)
                    } else {                                   // facula of the solar variant
                        acc[6][q].add(L * val(5));             // Bf (q_norm - fac_norm)
                        T w2 = (T)((double)L * fir_planck_ratio(A.lam[j], xc.temp, (double)A.t_norm_fac));
                        acc[4][q].add(w2 * val(1));            // Qf (q_norm)
                        acc[5][q].add(w2 * val(4));            // Af (fac_norm)
                    }
                }
            }
            __syncthreads();
        }
    }

    // --- outputs ----------------------------------------------------------------------
#pragma unroll
    for (int q = 0; q < FIR_PIX; ++q) {
        const int j = j0 + tid + q * FIR_THREADS;
        if (j >= n) continue;
        const long long o = (long long)l * A.out_stride + j;
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
            float2 is2 = A.cubes.spot_sed2[j], fs2 = A.cubes.fac_sed2[j];
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
            double is = A.cubes.spot_sed[j], fs = A.cubes.fac_sed[j];
            out0[o] = (OutT)(S - is * Qs - fs * Qf);   // flux
            out1[o] = (OutT)(Bs + Bf);                 // bconv
            out2[o] = (OutT)(S - is * As - fs * Af);   // tot
        }
    }
}

// --- phase integration: persistent, pipelined tile kernel -------------------------------
// true: a work unit's cube rows are staged in shared memory by TMA before it is applied;
// false: the apply loops read them from global memory (L1-cached), with no per-unit barrier
constexpr bool FIR_PP_STAGED = true;
constexpr int FIR_PP_WIN = FIR_PP_STAGED ? FIR_WIN : 4;   // staged values per cube row
// window buffers: unit u is staged in buffer u % NBUF, copied LEAD units ahead (when unit
// u - LEAD starts) into the buffer of unit u - NBUF, which every warp has released unless it
// lags NBUF - LEAD - 1 units behind the copying warp.  FP32 windows (18 KB): four buffers,
// copies two units ahead, so a copy's mbarrier and TMA latencies stay off the next unit's
// path; FP64 windows (37 KB, two blocks per SM): three buffers, one unit ahead.
template <typename T>
struct FirPPBuf {
    static constexpr int NBUF = FIR_PP_STAGED ? (sizeof(T) == 4 ? 4 : 3) : 2;
    static constexpr int LEAD = sizeof(T) == 4 ? 2 : 1;
    static_assert(!FIR_PP_STAGED || NBUF >= LEAD + 2, "a copy must not wait for the unit before it");
};
constexpr int FIR_PP_MINB = 2;   // resident blocks per SM the kernel is compiled for
constexpr int FIR_PP_EXC = 64;   // directly evaluated cells per staged batch
constexpr int FIR_FOLD = 8;          // work units per fold of the partial sums
// Shared memory of k_fir_pp: staged cube windows, two plan buffers, storage for the
// tiles that plan themselves, the direct cells' batch.
template <typename T>
struct FirPPSmem {
    Vec4<T> win[FirPPBuf<T>::NBUF][FIR_PP_WIN];
    __align__(16) unsigned char pb[2][FirPlanSlot<T>::BYTES];
    unsigned long long wbar[FirPPBuf<T>::NBUF], pbar[2];
    // released window buffers: every warp arrives once it has read a unit's window for
    // the last time, and the thread that copies a later unit into that buffer waits for
    // all of them first, so the warps need no block-wide barrier per unit
    unsigned long long ebar[FirPPBuf<T>::NBUF];
    FirPlanSt<T, 32, FIR_THREADS, FIR_THREADS> st;
    FirExcD<T> excd[FIR_PP_EXC];
    int wsum[FIR_THREADS / 32];
    int fail, nunit_sh;
    // followed by FirSeg seg[2 * seg_cap] (dynamic, 16-byte aligned)
};

template <typename T>
__host__ __device__ constexpr size_t fir_pp_smem_fixed() { return (sizeof(FirPPSmem<T>) + 15) & ~size_t(15); }

// The (phase, tile) pairs of the phases [r0, r0 + nr) (of the run list, when there is
// one) are walked tile by tile -- position v is tile v / nr of phase r0 + v % nr -- and
// block b takes the consecutive positions [b per, (b + 1) per): one block works through
// the phases of one tile, so consecutive phases read the same cube rows (L1 / L2).
// A tile's compact plan (k_fir_plan) is copied by TMA one tile ahead into the other plan
// buffer; the cube windows of its work units stream through NBUF buffers, LEAD units
// ahead (across the tile boundary, from the next tile's plan), each copy issued by lane 0
// of a rotating warp, so the copies' latencies overlap the arithmetic.  Tiles whose plan
// did not fit plan themselves.
// COMP: the output sums (per tile a pixel adds about 9 unit deficits, each rounded once)
// are compensated (Kahan) rather than plain FP32 sums.
// MULTI: the (phase, tile) pairs of many stars in one launch.  Star s has its own lists,
// prefix sums, plans and outputs (stars[s]); the stars share the wavelength grid and the
// typed cubes.  items[g] = (star, phase) for the nr visible phases of all stars, and the
// walk position v is tile v / nr of items[v % nr]; each block takes chunks of `chunk`
// consecutive positions, chunks b, b + G, b + 2G, ... (chunk = 0: one contiguous share).
template <typename T, bool COMP, bool MULTI>
__global__ void __launch_bounds__(FIR_THREADS, FIR_PP_MINB) k_fir_pp(const FirTileArgs A0, int ntile, int r0, int nr,
                                                        int ntot_all, const FirTileArgs *__restrict__ stars,
                                                        const int2 *__restrict__ items, int chunk) {
    constexpr int SLOT = FirPlanSlot<T>::BYTES;
    constexpr int NBUF = FirPPBuf<T>::NBUF, LEAD = FirPPBuf<T>::LEAD;
    extern __shared__ __align__(128) unsigned char pp_smem[];
    FirPPSmem<T> &sh = *reinterpret_cast<FirPPSmem<T> *>(pp_smem);
    FirSeg *segs = reinterpret_cast<FirSeg *>(pp_smem + fir_pp_smem_fixed<T>());
    __shared__ FirTileArgs star_sh;   // MULTI: the arguments of the star being walked
    const FirTileArgs &A = MULTI ? star_sh : A0;
    const int tid = threadIdx.x;
    const int G = gridDim.x;
    const int n = A0.n, n_eff = A0.n_eff;   // shared by every star
    if (tid == 0) {
        for (int q = 0; q < NBUF; ++q) {
            mbar_init(&sh.wbar[q], 1);
            mbar_init(&sh.ebar[q], FIR_THREADS / 32);
        }
        mbar_init(&sh.pbar[0], 1);
        mbar_init(&sh.pbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sh.fail = 0;
    }
    __syncthreads();

    // (phase, tile) index (phase * ntile + tile) of walk position v, and its star
    auto real = [&](int v) -> int {
        if (MULTI) return items[v % nr].y * ntile + v / nr;
        const int li = r0 + v % nr;
        return (A0.run_list ? A0.run_list[li] : li) * ntile + v / nr;
    };
    auto star_of = [&](int v) -> int { return MULTI ? items[v % nr].x : 0; };
    // plan record and size of walk position v (a star's plans: ntile x its lists slots, then
    // the sizes)
    auto plan_rec = [&](int v) -> const char * {
        const char *base = reinterpret_cast<const char *>(MULTI ? stars[star_of(v)].plan : A0.plan);
        return base + (size_t)real(v) * SLOT;
    };
    auto plan_size = [&](int v) -> unsigned {
        if (MULTI) {
            const FirTileArgs &S = stars[star_of(v)];
            const char *base = reinterpret_cast<const char *>(S.plan);
            return (unsigned)reinterpret_cast<const int *>(base + (size_t)ntile * S.n_lists_all * SLOT)[real(v)];
        }
        return (unsigned)reinterpret_cast<const int *>(reinterpret_cast<const char *>(A0.plan) +
                                                       (size_t)ntot_all * SLOT)[real(v)];
    };
    // this block's walk: positions [vb, ve) (chunk = 0), or chunks of `chunk` positions
    // taken round robin; step k of the walk is position pos(k), k < kend
    const int total = nr * ntile;
    int vb = 0, ve = 0, kend = 0;
    if (chunk <= 0) {
        const int per = (total + G - 1) / G;
        vb = min(total, (int)blockIdx.x * per);
        ve = min(total, vb + per);
        kend = ve - vb;
    } else {
        const int nchunk = (total + chunk - 1) / chunk;
        const int mine = nchunk > (int)blockIdx.x ? (nchunk - 1 - (int)blockIdx.x) / G + 1 : 0;
        kend = mine * chunk;
        if (mine > 0) {   // the last chunk of the walk may be short
            const int last = (int)blockIdx.x + (mine - 1) * G;
            kend -= (last + 1) * chunk - min(total, (last + 1) * chunk);
        }
    }
    auto pos = [&](int k) -> int {
        if (chunk <= 0) return vb + k;
        return ((int)blockIdx.x + (k / chunk) * G) * chunk + k % chunk;
    };
    // (thread 0) copy the plan of walk position v into plan buffer b; under the
    // failure-path test the block's first plan is expected but never copied
    auto issue_plan = [&](int v, int b, unsigned bytes, bool first = false) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&sh.pbar[b], bytes);
        if (!(first && A0.drop_plan)) bulk_g2s(&sh.pb[b][0], plan_rec(v), bytes, &sh.pbar[b]);
    };
    // (one thread) stage the interleaved rows of unit number u (buffer u % 3): pixels
    // [w0, w1) of the class's Vec4 row, one bulk copy (Vec4 elements are 16-byte multiples)
    auto issue_unit = [&](int u, const FirUnit &d) {
        // after a failed wait the block stops feeding the pipeline (no new expected bytes
        // on a buffer whose copy may never have landed) and leaves at the next barrier
        if (*reinterpret_cast<volatile int *>(&sh.fail)) return;
        const int b = u % NBUF;
        const unsigned bytes = (d.w1 > d.w0) ? (unsigned)(d.w1 - d.w0) * (unsigned)sizeof(Vec4<T>) : 0u;
        // buffer b last held unit u - NBUF: every warp must have released it
        if (u >= NBUF &&
            !mbar_wait_bounded(&sh.ebar[b], (unsigned)((u / NBUF - 1) & 1), A0.wait_limit)) {
            atomicExch(&sh.fail, 1);   // the unit is never copied: its readers' waits run out
            return;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&sh.wbar[b], bytes);
        if (bytes && !(A0.drop_unit && u == 0)) {
            // the typed cubes are the same for every star
            const Vec4<T> *row = reinterpret_cast<const Vec4<T> *>(A0.cubes.c[d.cls == CLS_SPOT ? 0 : 1]) +
                                 (long long)(d.key >> 1) * n;
            bulk_g2s(&sh.win[b][0], row + d.w0, bytes, &sh.wbar[b]);
        }
    };

    // compensated sums of the three outputs per pixel: flux, tot, bconv
    Acc<T, COMP> acc[3][FIR_PIX];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int q = 0; q < FIR_PIX; ++q) acc[a][q].zero();
    // the outputs' terms of one class at pixel j: flux S - I Q, tot S - I A, bconv B, with
    // I the class's continuum (spot or facula SED row); the products I Q and I A are
    // formed exactly inside fma (FP32: I as a float pair) and rounded once with S
    auto add_out = [&](int q, int j, bool spot, T S, T Q, T Aa, T B) {
        T f, t;
        if constexpr (sizeof(T) == 4) {
            const float2 w = (spot ? A.cubes.spot_sed2 : A.cubes.fac_sed2)[j];
            f = fmaf(-w.y, Q, fmaf(-w.x, Q, S));
            t = fmaf(-w.y, Aa, fmaf(-w.x, Aa, S));
        } else {
            const double w = (spot ? A.cubes.spot_sed : A.cubes.fac_sed)[j];
            f = fma(-w, Q, S);
            t = fma(-w, Aa, S);
        }
        acc[0][q].add(f);
        acc[1][q].add(t);
        acc[2][q].add(B);
    };

    // A unit's terms are summed in plain registers (part[slot][pixel]; slots per class:
    // spot S, Qs, As, Bs; facula S, Bf, Qf, Af) and folded into the compensated output
    // sums once per unit: a unit holds a few percent of a pixel's sum, so its FP32
    // partial carries rounding well below the compensated total's.
    T part[4][FIR_PIX];
    auto part_zero = [&]() {
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int q = 0; q < FIR_PIX; ++q) part[a][q] = (T)0;
    };
    auto part_fold = [&](int cls, int j0) {
        const bool spot = (cls == CLS_SPOT);
#pragma unroll
        for (int q = 0; q < FIR_PIX; ++q) {
            const int j = min(j0 + tid + q * FIR_THREADS, n - 1);   // pixels past n are not written
            if (spot) add_out(q, j, true, part[0][q], part[1][q], part[2][q], part[3][q]);
            else add_out(q, j, false, part[0][q], part[2][q], part[3][q], part[1][q]);
        }
    };
    // source rows of a unit, interleaved: the staged window (source pixel i at p[i + off])
    // or the class's row in global memory (off = 0)
    struct Src {
        const Vec4<T> *p;
        int off;
        bool staged;
    };
    auto cube_row = [&](int cls, int key) {
        return reinterpret_cast<const Vec4<T> *>(A.cubes.c[cls == CLS_SPOT ? 0 : 1]) + (long long)(key >> 1) * n;
    };
    auto src_of = [&](const Vec4<T> *W, const FirUnit &d) {
        Src sr;
        if (FIR_PP_STAGED) {
            sr.p = W;
            sr.off = d.off - d.w0;
            sr.staged = true;
        } else {
            sr.p = cube_row(d.cls, d.key);
            sr.off = 0;
            sr.staged = false;
        }
        return sr;
    };
    // groups [t_lo, t_hi) of unit d
    auto apply_groups = [&](const Src &sr, const FirUnit &d, const FirGrp<T> *grp, int t_lo, int t_hi, int j0,
                            int t_eff) {
        const int zv = d.key & 1;
        const bool fac = (d.cls != CLS_SPOT);
        const Vec4<T> *__restrict__ r = sr.p + sr.off;
        // one group at the thread's pixels; CHECKED: some pixels of the tile fall outside
        // [jlo, jhi] (tile edges, the grid's end), else none and no test is needed
        auto group_at = [&](auto checked_c, auto zv_c, const FirGrp<T> &gr, int jlo, int jhi, T b0, T b1, T bb) {
            constexpr bool CHECKED = decltype(checked_c)::value;
            constexpr bool ZV = decltype(zv_c)::value;
            const int m = gr.m;
#pragma unroll
            for (int q = 0; q < FIR_PIX; ++q) {
                const int dj = tid + q * FIR_THREADS;
                const int j = j0 + dj;
                if (CHECKED && (j < jlo || j > jhi)) continue;
                const int x = j + m;
                const Vec4<T> v0 = r[x];
                if constexpr (sizeof(T) == 4) {
                    // FP32: the four rows as two packed pairs (x, y) and (z, w), each lane
                    // rounded as the scalar FMA would be
                    if (ZV) {   // single tap: w == 0
                        soap_fma2(part[0][q], part[1][q], gr.a0, gr.a0, v0.x, v0.y);
                        soap_fma2(part[2][q], part[3][q], b0, b0, v0.z, v0.w);
                        continue;
                    }
                    const Vec4<T> v1 = r[x + 1];
                    const float fdj = (float)dj;
                    float c0 = gr.a0, c0b = gr.a0, c1 = gr.a1, c1b = gr.a1;
                    float e0 = b0, e0b = b0, e1 = b1, e1b = b1;
                    soap_fma2(c0, c0b, -gr.b, -gr.b, fdj, fdj);
                    soap_fma2(c1, c1b, gr.b, gr.b, fdj, fdj);
                    soap_fma2(e0, e0b, -bb, -bb, fdj, fdj);
                    soap_fma2(e1, e1b, bb, bb, fdj, fdj);
                    soap_fma2(part[0][q], part[1][q], c0, c0b, v0.x, v0.y);
                    soap_fma2(part[0][q], part[1][q], c1, c1b, v1.x, v1.y);
                    soap_fma2(part[2][q], part[3][q], e0, e0b, v0.z, v0.w);
                    soap_fma2(part[2][q], part[3][q], e1, e1b, v1.z, v1.w);
                } else {
                    if (ZV) {   // single tap: w == 0
                        part[0][q] = fma(gr.a0, v0.x, part[0][q]);
                        part[1][q] = fma(gr.a0, v0.y, part[1][q]);
                        part[2][q] = fma(b0, v0.z, part[2][q]);
                        part[3][q] = fma(b0, v0.w, part[3][q]);
                        continue;
                    }
                    const Vec4<T> v1 = r[x + 1];
                    const T fdj = (T)dj;
                    const T c0 = fma(-gr.b, fdj, gr.a0), c1 = fma(gr.b, fdj, gr.a1);
                    const T e0 = fma(-bb, fdj, b0), e1 = fma(bb, fdj, b1);
                    // two chained FMAs per row (no separate product and sum)
                    part[0][q] = fma(c1, v1.x, fma(c0, v0.x, part[0][q]));
                    part[1][q] = fma(c1, v1.y, fma(c0, v0.y, part[1][q]));
                    part[2][q] = fma(e1, v1.z, fma(e0, v0.z, part[2][q]));
                    part[3][q] = fma(e1, v1.w, fma(e0, v0.w, part[3][q]));
                }
            }
        };
        using yes = std::integral_constant<bool, true>;
        using no = std::integral_constant<bool, false>;
        for (int t = t_lo; t < t_hi; ++t) {
            const FirGrp<T> gr = grp[t];
            if (!gr.ok) continue;
            const int m = gr.m;
            const int jlo = max(j0, -m);
            const int jhi = zv ? j0 + t_eff - 1 : min(j0 + t_eff - 1, n_eff - 2 - m);
            // facula slots 2, 3 carry the (1 + LB) L weights, spot slots 2, 3 the L weights
            const T b0 = fac ? gr.a0w : gr.a0, b1 = fac ? gr.a1w : gr.a1, bb = fac ? gr.bw : gr.b;
            const bool inside = (jlo <= j0) && (jhi >= j0 + FIR_TILE - 1);   // uniform for the block
            if (zv) {
                if (inside) group_at(no(), yes(), gr, jlo, jhi, b0, b1, bb);
                else group_at(yes(), yes(), gr, jlo, jhi, b0, b1, bb);
            } else {
                if (inside) group_at(no(), no(), gr, jlo, jhi, b0, b1, bb);
                else group_at(yes(), no(), gr, jlo, jhi, b0, b1, bb);
            }
        }
    };
    // wrap cells exc[0, ne) of unit d (per-cell lerp; with staged rows, pixels whose owner
    // falls outside the window read the row in global memory)
    auto apply_exc = [&](const Src &sr, const FirUnit &d, const FirExcW<T> *exc, int ne, int j0) {
        const int cls = d.cls;
        const bool fac = (cls != CLS_SPOT);
        // one wrap cell at the thread's pixels; CHECKED: a pixel may lie past n_eff or
        // read a source outside [0, n_eff - 2] or outside the staged window; else none can
        auto cell_at = [&](auto checked_c, const FirExcW<T> &xc, T w23) {
            constexpr bool CHECKED = decltype(checked_c)::value;
#pragma unroll
            for (int q = 0; q < FIR_PIX; ++q) {
                const int dj = tid + q * FIR_THREADS;
                const int j = j0 + dj;
                if (CHECKED && j >= n_eff) continue;
                T wd = xc.phi + xc.dlt * (T)dj;
                int i = xc.i0 + dj;
                if (wd >= (T)1) { wd -= (T)1; i += 1; }
                else if (wd < (T)0) { wd += (T)1; i -= 1; }
                if (CHECKED && (i < 0 || i > n_eff - 2)) continue;
                const bool inwin = !CHECKED || !sr.staged || ((i >= d.w0) && (i + 1 < d.w1));
                Vec4<T> s0, s1;
                if (inwin) {
                    s0 = sr.p[i + sr.off];
                    s1 = sr.p[i + 1 + sr.off];
                } else {
                    const Vec4<T> *rowp = cube_row(cls, d.key);
                    s0 = rowp[i];
                    s1 = rowp[i + 1];
                }
                if constexpr (sizeof(T) == 4) {   // packed pairs (x, y) and (z, w)
                    float gx = s1.x, gy = s1.y, gz = s1.z, gw = s1.w;
                    soap_sub2(gx, gy, s0.x, s0.y);
                    soap_sub2(gz, gw, s0.z, s0.w);
                    float ux = s0.x, uy = s0.y, uz = s0.z, uw = s0.w;
                    soap_fma2(ux, uy, gx, gy, wd, wd);
                    soap_fma2(uz, uw, gz, gw, wd, wd);
                    soap_fma2(part[0][q], part[1][q], xc.L, xc.L, ux, uy);
                    soap_fma2(part[2][q], part[3][q], w23, w23, uz, uw);
                } else {
                    part[0][q] = fma(xc.L, fma(s1.x - s0.x, wd, s0.x), part[0][q]);
                    part[1][q] = fma(xc.L, fma(s1.y - s0.y, wd, s0.y), part[1][q]);
                    part[2][q] = fma(w23, fma(s1.z - s0.z, wd, s0.z), part[2][q]);
                    part[3][q] = fma(w23, fma(s1.w - s0.w, wd, s0.w), part[3][q]);
                }
            }
        };
        // the sources of a cell span [i0 - 1, i0 + FIR_TILE] over the tile
        const bool full = (j0 + FIR_TILE <= n_eff);
        for (int e = 0; e < ne; ++e) {
            const FirExcW<T> xc = exc[e];
            const T w23 = fac ? xc.w2 : xc.L;
            const int ilo = xc.i0 - 1, ihi = xc.i0 + FIR_TILE;
            const bool inside = full && ilo >= 0 && ihi <= n_eff - 2 &&
                                (!sr.staged || (ilo >= d.w0 && ihi + 1 < d.w1));   // uniform for the block
            if (inside) cell_at(std::integral_constant<bool, false>(), xc, w23);
            else cell_at(std::integral_constant<bool, true>(), xc, w23);
        }
    };
    // wait for unit u's rows (every thread; a timeout sets the block's fail flag)
    // wait for unit u's rows.  Planned tiles: every thread for itself, with no barrier;
    // a timeout sets the block's fail flag, the thread goes on with the buffer as it is
    // (its reads stay inside the window) and the block leaves together at the next tile's
    // barrier.  Tiles that plan themselves (block-wide steps with barriers): the barrier
    // here, and the block leaves together at once.
    auto wait_unit = [&](int u) {
        if (!mbar_wait_bounded(&sh.wbar[u % NBUF], (unsigned)((u / NBUF) & 1), A0.wait_limit))
            atomicExch(&sh.fail, 1);
    };
    auto wait_unit_sync = [&](int u) {
        wait_unit(u);
        __syncthreads();
        return sh.fail == 0;
    };
    // (every thread) done with unit u's window: one arrival per warp
    auto release_unit = [&](int u) {
        __syncwarp();
        if ((tid & 31) == 0) mbar_arrive(&sh.ebar[u % NBUF]);
    };

    // walk steps [0, kend)
    if (tid == 0) {
        if (kend > 0) issue_plan(pos(0), 0, plan_size(pos(0)), true);
        if (kend > 1) issue_plan(pos(1), 1, plan_size(pos(1)));
    }
    int ucount = 0;        // units staged and applied so far (window buffer ucount % NBUF)
    // a planned tile's units [ahead_lo, LEAD) were copied during the previous tile (the
    // copying thread's test, repeated by every thread); the others are copied at its start
    int ahead_lo = LEAD;
    int k = 0;
    int bad = 0;
    int cur_star = -1;     // MULTI: the star whose arguments star_sh holds
    unsigned next_plan_bytes = 0;   // (thread 0) size of the plan of step k + 1, read during step k - 1
    for (; k < kend && !bad; ++k) {
        const int v = pos(k);
        const int pbuf = k & 1;
        // size of the plan issued at the end of this tile, read early (its latency hides
        // behind the tile's work)
        const unsigned next_bytes = (tid == 0 && k + 2 < kend) ? plan_size(pos(k + 2)) : 0u;
        if (MULTI) {
            const int s_v = star_of(v);   // uniform for the block
            if (s_v != cur_star) {
                __syncthreads();   // every thread is done with the previous star's arguments
                constexpr int WORDS = (int)(sizeof(FirTileArgs) / sizeof(int));
                static_assert(sizeof(FirTileArgs) % sizeof(int) == 0, "FirTileArgs copied as words");
                const int *src = reinterpret_cast<const int *>(stars + s_v);
                int *dst = reinterpret_cast<int *>(&star_sh);
                for (int w = tid; w < WORDS; w += FIR_THREADS) dst[w] = src[w];
                cur_star = s_v;
            }
        }
        if (!mbar_wait_bounded(&sh.pbar[pbuf], (unsigned)((k >> 1) & 1), A0.wait_limit)) atomicExch(&sh.fail, 1);
        __syncthreads();   // the one barrier of a planned tile: the block leaves together on a failure
        if (sh.fail) {
            bad = 1;
            break;
        }
        // every thread is done with step k - 1, so its plan buffer takes the plan of step k + 1
        if (tid == 0 && k >= 1 && k + 1 < kend) issue_plan(pos(k + 1), pbuf ^ 1, next_plan_bytes);
        T *out0 = reinterpret_cast<T *>(A.out0);
        T *out1 = reinterpret_cast<T *>(A.out1);
        T *out2 = reinterpret_cast<T *>(A.out2);
        const int tr = real(v);
        const int l = tr / ntile, j0 = (tr - l * ntile) * FIR_TILE;
        const int t_eff = min(FIR_TILE, n_eff - j0);
        const long long lbase = (long long)l * A.gm;
        const int *cn = A.counts + 4 * l;
        const unsigned char *rec = sh.pb[pbuf];
        const int4 hdr = *reinterpret_cast<const int4 *>(rec);
        const int lo = ahead_lo;
        ahead_lo = LEAD;
        if (t_eff > 0 && hdr.w) {
            // --- planned tile ------------------------------------------------------------
            const int nb = hdr.x;
            const FirPlanLayout<T> L(hdr.x, hdr.y, hdr.z);
            const FirUnit *units = reinterpret_cast<const FirUnit *>(rec + L.o_unit);
            const int *ut = reinterpret_cast<const int *>(rec + L.o_ut);
            const int *woff = reinterpret_cast<const int *>(rec + L.o_woff);
            const FirGrp<T> *grp = reinterpret_cast<const FirGrp<T> *>(rec + L.o_grp);
            const FirExcW<T> *exc = reinterpret_cast<const FirExcW<T> *>(rec + L.o_exc);
            int nfold = 0;   // units summed in part[] since the last fold
            // unit u is copied by lane 0 of warp u % 8: the copies' mbarrier latencies are
            // spread over the warps instead of holding back one of them
            if (FIR_PP_STAGED)
                for (int i = 0; i < min(lo, nb); ++i)
                    if (tid == ((ucount + i) % FIR_WARPS) * 32) issue_unit(ucount + i, units[i]);
            for (int ui = 0; ui < nb; ++ui) {
                const int u = ucount;
                if (!FIR_PP_STAGED) {   // rows read from global memory: no staging, no barrier
                    const FirUnit d = units[ui];
                    const Src sr = src_of(nullptr, d);
                    part_zero();
                    apply_groups(sr, d, grp, ut[ui], ut[ui + 1], j0, t_eff);
                    const int e_lo = woff[ut[ui]], e_hi = woff[ut[ui + 1]];
                    apply_exc(sr, d, exc + e_lo, e_hi - e_lo, j0);
                    part_fold(d.cls, j0);
                    continue;
                }
                // unit u + LEAD: this tile's unit ui + LEAD, else the next tile's unit
                // ui + LEAD - nb, from its plan
                if (tid == ((u + LEAD) % FIR_WARPS) * 32) {
                    const int i2 = ui + LEAD;
                    if (i2 < nb) {
                        issue_unit(u + LEAD, units[i2]);
                    } else if (k + 1 < kend) {
                        if (mbar_wait_bounded(&sh.pbar[pbuf ^ 1], (unsigned)(((k + 1) >> 1) & 1), A0.wait_limit)) {
                            const unsigned char *rn = sh.pb[pbuf ^ 1];
                            const int4 hn = *reinterpret_cast<const int4 *>(rn);
                            const int tnr = real(pos(k + 1));
                            const int ln = tnr / ntile, jn = (tnr - ln * ntile) * FIR_TILE;
                            if (hn.w && i2 - nb < hn.x && jn < n_eff) {
                                const FirPlanLayout<T> Ln(hn.x, hn.y, hn.z);
                                issue_unit(u + LEAD, reinterpret_cast<const FirUnit *>(rn + Ln.o_unit)[i2 - nb]);
                            }
                        } else {
                            atomicExch(&sh.fail, 1);   // the block leaves at the next tile's barrier
                        }
                    }
                }
                wait_unit(u);
                const FirUnit d = units[ui];
                const Src sr = src_of(sh.win[u % NBUF], d);
                if (nfold == 0) part_zero();
                apply_groups(sr, d, grp, ut[ui], ut[ui + 1], j0, t_eff);
                const int e_lo = woff[ut[ui]], e_hi = woff[ut[ui + 1]];
                apply_exc(sr, d, exc + e_lo, e_hi - e_lo, j0);
                // the partial sums cover up to FIR_FOLD units of one class
                if (++nfold == FIR_FOLD || ui + 1 == nb || units[ui + 1].cls != d.cls) {
                    part_fold(d.cls, j0);
                    nfold = 0;
                }
                release_unit(u);
                ++ucount;
            }
            if (k + 1 < kend) ahead_lo = max(0, LEAD - nb);
        } else if (t_eff > 0) {
            // --- tile that plans itself, batch by batch ----------------------------------
            const int nsg = A.nseg[2 * l] + A.nseg[2 * l + 1];
            const int nunit = fir_segments<MODE_PHASE, FIR_THREADS>(A, l, j0, t_eff, segs, nsg, &sh.nunit_sh);
            auto &st = sh.st;
            const double *sl = A.list_dlt + lbase;
            for (int ub = 0; ub < nunit && !bad;) {
                fir_plan_batch<T, MODE_PHASE, FIR_THREADS>(A, l, j0, t_eff, segs, nsg, nunit, sl, st, ub, sh.wsum);
                const int nb = st.nb;
                for (int ui = 0; ui < nb; ++ui) {
                    const int u = ucount;
                    if (FIR_PP_STAGED) {
                        if (tid == 0) {
                            if (ui == 0) issue_unit(u, st.unit[0]);
                            if (ui + 1 < nb) issue_unit(u + 1, st.unit[ui + 1]);
                        }
                        if (!wait_unit_sync(u)) {
                            bad = 1;
                            break;
                        }
                    }
                    const FirUnit d = st.unit[ui];
                    const Src sr = src_of(sh.win[u % NBUF], d);
                    part_zero();
                    apply_groups(sr, d, st.grp, st.ut[ui], st.ut[ui + 1], j0, t_eff);
                    const int e_lo = st.woff[st.ut[ui]], e_hi = st.woff[st.ut[ui + 1]];
                    for (int cb = e_lo; cb < e_hi; cb += FirPlanSt<T, 32, FIR_THREADS, FIR_THREADS>::NE) {
                        const int ce = min(e_hi, cb + FirPlanSt<T, 32, FIR_THREADS, FIR_THREADS>::NE);
                        const FirExcW<T> *ex = st.excw + cb;
                        if (e_hi > FirPlanSt<T, 32, FIR_THREADS, FIR_THREADS>::NE) {   // refill this chunk
                            __syncthreads();
                            fir_fill_exc<T, FIR_THREADS>(A, l, j0, st, cb, ce, cb);
                            __syncthreads();
                            ex = st.excw;
                        }
                        apply_exc(sr, d, ex, ce - cb, j0);
                    }
                    part_fold(d.cls, j0);
                    __syncthreads();
                    if (FIR_PP_STAGED) release_unit(u);
                    ++ucount;
                }
                ub += nb;
            }
            if (bad) break;
        }
        if (bad) break;
        // --- directly evaluated cells (spots of non-integral temperature, solar faculae)
        if (t_eff > 0 && cn[2] > 0) {
            const int c_start = cn[0] + cn[1], c_cnt = cn[2];
            for (int b0 = 0; b0 < c_cnt; b0 += FIR_PP_EXC) {
                const int nbd = min(FIR_PP_EXC, c_cnt - b0);
                if (tid < nbd) {
                    const int cell = A.list_cell[lbase + c_start + b0 + tid];
                    FirExcD<T> x;
                    cell_pos<T>(j0, A.geo, A.geo32, cell, x.i0, x.phi, x.dlt, x.L, x.w2);
                    const CellGeo &gg = A.geo[cell];
                    x.row = gg.row;
                    x.zero_v = gg.zero_v;
                    const double2 ax = A.list_aux[lbase + c_start + b0 + tid];
                    x.temp = ax.x;
                    x.kind = bits_is_zero(ax.y) ? 0 : 1;
                    sh.excd[tid] = x;
                }
                __syncthreads();
                for (int e = 0; e < nbd; ++e) {
                    const FirExcD<T> xc = sh.excd[e];
                    // the class's interleaved row: spot (q_sed, q_norm, spot_norm, -),
                    // facula (q_sed, -, q_norm, fac_norm)
                    const Vec4<T> *rowp = cube_row(xc.kind == 0 ? CLS_SPOT : CLS_FAC, 2 * xc.row);
#pragma unroll
                    for (int q = 0; q < FIR_PIX; ++q) {
                        const int dj = tid + q * FIR_THREADS;
                        const int j = j0 + dj;
                        if (j >= n_eff) continue;
                        long long i;
                        T w;
                        if (xc.zero_v) {
                            i = j;
                            w = (T)0;
                        } else {
                            T wd = xc.phi + xc.dlt * (T)dj;
                            i = (long long)xc.i0 + dj;
                            if (wd >= (T)1) { wd -= (T)1; i += 1; }
                            else if (wd < (T)0) { wd += (T)1; i -= 1; }
                            if (i < 0 || i > n_eff - 2) continue;
                            w = wd;
                        }
                        const Vec4<T> a = rowp[i];
                        Vec4<T> v = a;
                        if (!xc.zero_v) {
                            const Vec4<T> b = rowp[i + 1];
                            v.x = a.x + (b.x - a.x) * w;
                            v.y = a.y + (b.y - a.y) * w;
                            v.z = a.z + (b.z - a.z) * w;
                            v.w = a.w + (b.w - a.w) * w;
                        }
                        const T Lc = xc.L;
                        if (xc.kind == 0) {
                            T Lq = (T)((double)Lc * fir_planck_ratio(A.lam[j], xc.temp, (double)(int)xc.temp));
                            add_out(q, j, true, Lc * v.x, Lq * v.y, Lq * v.z, Lc * v.w);
                        } else {
                            T w2 = (T)((double)Lc * fir_planck_ratio(A.lam[j], xc.temp, (double)A.t_norm_fac));
                            add_out(q, j, false, Lc * v.x, w2 * v.z, w2 * v.w, Lc * v.y);
                        }
                    }
                }
                __syncthreads();
            }
        }
        // --- outputs; accumulators reset for the next tile ---------------------------------
#pragma unroll
        for (int q = 0; q < FIR_PIX; ++q) {
            const int j = j0 + tid + q * FIR_THREADS;
            if (j < n) {
                const long long o = (long long)l * A.out_stride + j;
                if (j >= n_eff) {
                    out0[o] = (T)0;
                    out1[o] = (T)0;
                    out2[o] = (T)0;
                } else {
                    // the compensated sums, rounded once to the output type
                    out0[o] = (T)(acc[0][q].s - acc[0][q].c);   // flux
                    out1[o] = (T)(acc[2][q].s - acc[2][q].c);   // bconv
                    out2[o] = (T)(acc[1][q].s - acc[1][q].c);   // tot
                }
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) acc[a][q].zero();
        }
        next_plan_bytes = next_bytes;
    }
    // a wait that ran out in the last step (no tile barrier after it)
    __syncthreads();
    if (sh.fail) bad = 1;
    if (bad && tid == 0) {
        // a copy did not land in time: record it and give the copies possibly in flight a
        // bounded wait before leaving
        atomicExch(A0.status, FIR_ST_WAIT);
        if (FIR_PP_STAGED) {
            for (int i = 0; i < LEAD; ++i)
                mbar_wait_bounded(&sh.wbar[(ucount + i) % NBUF], (unsigned)(((ucount + i) / NBUF) & 1), A0.wait_limit);
        }
        mbar_wait_bounded(&sh.pbar[k & 1], (unsigned)((k >> 1) & 1), A0.wait_limit);
        mbar_wait_bounded(&sh.pbar[(k + 1) & 1], (unsigned)(((k + 1) >> 1) & 1), A0.wait_limit);
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// outputs [0, n) of the phases zero_list[0, count) set to zero (phases without a visible
// region: no active cell, so their deficit spectra are zero)
template <typename T>
__global__ void k_fir_zero(int n, const int *__restrict__ zero_list, T *out0, T *out1, T *out2, long long out_stride) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const long long o = (long long)zero_list[blockIdx.y] * out_stride + j;
    out0[o] = (T)0;
    out1[o] = (T)0;
    out2[o] = (T)0;
}

__global__ void k_pair_rows(int n, const double *__restrict__ a, const double *__restrict__ b, float2 *pa, float2 *pb) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float ah = (float)a[i], bh = (float)b[i];
    pa[i] = make_float2(ah, (float)(a[i] - (double)ah));
    pb[i] = make_float2(bh, (float)(b[i] - (double)bh));
}

namespace {

// workspace layout of the FAST forms
struct FirLayout {
    enum {
        GEO, GEO32, CUBE0, SED2A = CUBE0 + 6, SED2B, K1A, K1B, K2A, K2B, VA, VB, SORT_TMP, LCELL, LDLT, LAUX,
        COUNTS, PRE, SEGS, NSEG, PLAN, NSLOT
    };
    size_t off[NSLOT] = {0};
    size_t total = 0;
    int seg_cap = 0;
    long long pre_stride = 0, pre_comp = 0;
};

// typed_external: the typed cubes live elsewhere (shared by several stars), no slots here
FirLayout fir_layout(int form, int n, int n_mu, long long gm, int ncube, int n_lists, bool typed_external = false) {
    FirLayout L;
    size_t tsz = (form == SOAPGB_FAST32) ? 4 : 8;
    size_t sz[FirLayout::NSLOT] = {0};
    sz[FirLayout::GEO] = sizeof(CellGeo) * (size_t)gm;
    sz[FirLayout::GEO32] = sizeof(CellGeo32) * (size_t)gm;
    // QUIET: one cube of T; PHASE (ncube 6): the two classes' interleaved rows (4 x T)
    for (int q = 0; q < 6; ++q)
        sz[FirLayout::CUBE0 + q] = typed_external ? 0
                                   : (ncube == 1 && q == 0) ? tsz * (size_t)n * n_mu
                                   : (ncube == 6 && q < 2)  ? 4 * tsz * (size_t)n * n_mu
                                                            : 0;
    sz[FirLayout::SED2A] = sz[FirLayout::SED2B] = typed_external ? 0 : sizeof(float2) * (size_t)n;
    sz[FirLayout::K1A] = sz[FirLayout::K1B] = sizeof(unsigned long long) * (size_t)gm;
    sz[FirLayout::K2A] = sz[FirLayout::K2B] = sizeof(unsigned) * (size_t)gm;
    sz[FirLayout::VA] = sz[FirLayout::VB] = sizeof(int) * (size_t)gm;
    sz[FirLayout::SORT_TMP] = soapgb::fir_sort_temp_bytes(gm);
    sz[FirLayout::LCELL] = sizeof(int) * (size_t)gm * n_lists;
    sz[FirLayout::LDLT] = sizeof(double) * (size_t)gm * n_lists;
    sz[FirLayout::LAUX] = (ncube == 6) ? sizeof(double2) * (size_t)gm * n_lists : 0;
    sz[FirLayout::COUNTS] = sizeof(int) * 4 * (size_t)n_lists;
    L.pre_stride = gm + 2;
    L.pre_comp = L.pre_stride * n_lists;
    sz[FirLayout::PRE] = sizeof(double) * 6 * (size_t)L.pre_comp;
    L.seg_cap = 2 * n_mu;
    sz[FirLayout::SEGS] = sizeof(int2) * 2 * (size_t)L.seg_cap * n_lists;
    sz[FirLayout::NSEG] = sizeof(int) * 2 * (size_t)n_lists;
    // precomputed tile plans of the phase integration
    const size_t ntile = ((size_t)n + FIR_TILE - 1) / FIR_TILE;
    if (ncube == 6)
        sz[FirLayout::PLAN] = ntile * n_lists *
                              ((form == SOAPGB_FAST32) ? (size_t)FirPlanSlot<float>::BYTES + sizeof(int)
                                                       : (size_t)FirPlanSlot<double>::BYTES + sizeof(int));
    size_t t = 0;
    for (int s = 0; s < FirLayout::NSLOT; ++s) {
        L.off[s] = t;
        t += align256(sz[s]);
    }
    L.total = t;
    return L;
}

}  // namespace

FirPlanSizes fir_plan_sizes(int form, int n, int n_mu, long long gm, bool phase, int n_lists, bool typed_external) {
    FirPlanSizes p;
    if (form == SOAPGB_PLAIN64) return p;
    p.bytes = fir_layout(form, n, n_mu, gm, phase ? 6 : 1, n_lists > 0 ? n_lists : 1, typed_external).total;
    return p;
}

size_t fir_typed_bytes(int form, int n, int n_mu) {
    const size_t tsz = (form == SOAPGB_FAST32) ? 4 : 8;
    return 2 * align256(4 * tsz * (size_t)n * n_mu) + 2 * align256(sizeof(float2) * (size_t)n);
}

// the typed cubes of the phase integration: the two classes' interleaved rows (Vec4 of
// T per pixel) and, in the FP32 form, the continuum rows as float pairs
static int typed_cubes_into(soapgb_ctx *ctx, int form, int n, const soapgb_cubes &c, void *const dst[2],
                            float2 *sed2a, float2 *sed2b) {
    const int n_mu = c.n_mu;
    const size_t cube_elems = (size_t)n * n_mu;
    auto al16 = [](const void *p) { return ((uintptr_t)p & 15) == 0; };
    const bool paired = (form == SOAPGB_FAST32) && (cube_elems % 2 == 0) && al16(c.q_sed) && al16(c.q_norm) &&
                        al16(c.spot_norm) && al16(c.fac_norm);
    if (paired) {
        const long long n2 = (long long)(cube_elems / 2);
        // short blocks (two steps per thread): SMs free up quickly for the
        // higher-priority geometry kernels that run beside this one
        const int nblk = (int)std::max<long long>(1, (n2 + 511) / 512);
        SOAP_TRACED(ctx, "cube_types",
                    k_cube_types32<<<nblk, 256, 0, ctx->stream>>>(
                        n2, (const double2 *)c.q_sed, (const double2 *)c.q_norm, (const double2 *)c.spot_norm,
                        (const double2 *)c.fac_norm, (float4 *)dst[0], (float4 *)dst[1]));
        SOAP_LAUNCHED(ctx);
    } else if (form == SOAPGB_FAST32) {
        SOAP_TRACED(ctx, "cube_types", k_cube_rows<float><<<grid_for(ctx, cube_elems, 256), 256, 0, ctx->stream>>>(
                                           cube_elems, c.q_sed, c.q_norm, c.spot_norm, c.fac_norm,
                                           (float4 *)dst[0], (float4 *)dst[1]));
        SOAP_LAUNCHED(ctx);
    } else {
        SOAP_TRACED(ctx, "cube_types", k_cube_rows<double><<<grid_for(ctx, cube_elems, 256), 256, 0, ctx->stream>>>(
                                           cube_elems, c.q_sed, c.q_norm, c.spot_norm, c.fac_norm,
                                           (soap_double4 *)dst[0], (soap_double4 *)dst[1]));
        SOAP_LAUNCHED(ctx);
    }
    if (form == SOAPGB_FAST32) {
        k_pair_rows<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, c.spot_sed, c.fac_sed, sed2a, sed2b);
        SOAP_LAUNCHED(ctx);
    }
    return SOAPGB_OK;
}

void fir_typed_layout(int form, int n, int n_mu, char *dst, const soapgb_cubes &c, FirTyped *out) {
    const size_t tsz = (form == SOAPGB_FAST32) ? 4 : 8;
    const size_t cb = align256(4 * tsz * (size_t)n * n_mu);
    for (int q = 0; q < 6; ++q) out->c[q] = nullptr;
    out->c[0] = dst;
    out->c[1] = dst + cb;
    out->spot_sed = c.spot_sed;
    out->fac_sed = c.fac_sed;
    out->spot_sed2 = dst + 2 * cb;
    out->fac_sed2 = dst + 2 * cb + align256(sizeof(float2) * (size_t)n);
}

int fir_typed_cubes(soapgb_ctx *ctx, int form, int n, const soapgb_cubes &c, char *dst, FirTyped *out) {
    fir_typed_layout(form, n, c.n_mu, dst, c, out);
    void *d[2] = {const_cast<void *>(out->c[0]), const_cast<void *>(out->c[1])};
    return typed_cubes_into(ctx, form, n, c, d, (float2 *)const_cast<void *>(out->spot_sed2),
                            (float2 *)const_cast<void *>(out->fac_sed2));
}

static int fir_prepare(soapgb_ctx *ctx, const double *wave, int n_eff, double step, long long gm, const double *delta,
                       const double *limb, const double *lb, const int *region, int n_mu, CellGeo *geo,
                       CellGeo32 *geo32, double *lambda0) {
    if (!(*lambda0 > 0.0)) {   // not given by the caller: read it from the device
        SOAP_CUDA(ctx, cudaMemcpyAsync(lambda0, wave, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    k_check_uniform<<<grid_for(ctx, n_eff, 256), 256, 0, ctx->stream>>>(n_eff, wave, step, ctx->d_status);
    SOAP_LAUNCHED(ctx);
    SOAP_TRACED(ctx, "cell_geo", k_cell_geo<<<grid_for(ctx, gm, 256), 256, 0, ctx->stream>>>(gm, delta, limb, lb, region, n_mu, *lambda0, step, geo,
                                                                geo32, ctx->d_status));
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}

// velocity-ordered cell lists, prefix sums and segments for n_lists lists
static int fir_lists(soapgb_ctx *ctx, const FirLayout &L, char *ws, long long gm, int n_lists, const double *temp,
                     const double *bi, int solar, const FirPhaseArgs *boxes = nullptr) {
    const CellGeo *geo = (const CellGeo *)(ws + L.off[FirLayout::GEO]);
    if (boxes && boxes->box_cap > 0) {
        // phases sort their own active cells: no cell order needed
        int *lcell = (int *)(ws + L.off[FirLayout::LCELL]);
        double *ldlt = (double *)(ws + L.off[FirLayout::LDLT]);
        double2 *laux = (double2 *)(ws + L.off[FirLayout::LAUX]);
        int *counts = (int *)(ws + L.off[FirLayout::COUNTS]);
        const int cap = boxes->box_cap;
        const size_t smem = (size_t)cap * 3 * sizeof(unsigned long long);
        SOAP_CUDA(ctx, cudaFuncSetAttribute(k_fir_slists, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const soapgb_activity *act = boxes->act;
        SOAP_TRACED(ctx, "fir_lists",
                    k_fir_slists<<<n_lists, FIR_SLIST_THREADS, smem, ctx->stream>>>(
                        boxes->grid, 2. / boxes->grid, boxes->table, boxes->reg_off, act->t_star, act->t_diff_spot,
                        act->t_diff_fac, solar, cap, geo, lcell, ldlt, laux, counts, ctx->d_status));
        SOAP_LAUNCHED(ctx);
        double *pre = (double *)(ws + L.off[FirLayout::PRE]);
        int2 *segs = (int2 *)(ws + L.off[FirLayout::SEGS]);
        int *nseg = (int *)(ws + L.off[FirLayout::NSEG]);
        SOAP_TRACED(ctx, "fir_prefix", k_fir_prefix<<<dim3(n_lists, 2), 256, 0, ctx->stream>>>(
                                           gm, counts, lcell, geo, pre, L.pre_stride, L.pre_comp, segs, nseg,
                                           L.seg_cap, ctx->d_status));
        SOAP_LAUNCHED(ctx);
        return SOAPGB_OK;
    }
    auto *k1a = (unsigned long long *)(ws + L.off[FirLayout::K1A]);
    auto *k1b = (unsigned long long *)(ws + L.off[FirLayout::K1B]);
    auto *k2a = (unsigned *)(ws + L.off[FirLayout::K2A]);
    auto *k2b = (unsigned *)(ws + L.off[FirLayout::K2B]);
    int *va = (int *)(ws + L.off[FirLayout::VA]);
    int *vb = (int *)(ws + L.off[FirLayout::VB]);
    void *tmp = ws + L.off[FirLayout::SORT_TMP];
    size_t tmp_bytes = soapgb::fir_sort_temp_bytes(gm);
    int g = grid_for(ctx, gm, 256);
    k_sort_keys1<<<g, 256, 0, ctx->stream>>>(gm, geo, k1a, va);
    SOAP_LAUNCHED(ctx);
    int rc;
    {
        soapgb::TraceScope ts(ctx, "cell_sort");
        rc = soapgb::fir_sort_u64(ctx, gm, k1a, k1b, va, vb, tmp, tmp_bytes);
    }
    if (rc) return rc;
    k_sort_keys2<<<g, 256, 0, ctx->stream>>>(gm, geo, vb, k2a);
    SOAP_LAUNCHED(ctx);
    {
        soapgb::TraceScope ts(ctx, "cell_sort");
        rc = soapgb::fir_sort_u32(ctx, gm, k2a, k2b, vb, va, 14, tmp, tmp_bytes);   // stable: dlt order kept per bin
    }
    if (rc) return rc;
    int *lcell = (int *)(ws + L.off[FirLayout::LCELL]);
    double *ldlt = (double *)(ws + L.off[FirLayout::LDLT]);
    double2 *laux = (double2 *)(ws + L.off[FirLayout::LAUX]);
    int *counts = (int *)(ws + L.off[FirLayout::COUNTS]);
    if (boxes) {
        // phases without maps: lists from the region boxes
        if (gm > fir_box_lists_max_gm())
            return set_error(ctx, SOAPGB_ERR_ARG, "box lists: grid of %lld cells above %lld", gm, fir_box_lists_max_gm());
        int *rank = vb;   // free after the second sort
        SOAP_TRACED(ctx, "fir_rank", k_fir_rank<<<g, 256, 0, ctx->stream>>>(gm, va, rank));
        SOAP_LAUNCHED(ctx);
        const size_t smem = fir_blists_smem(gm);
        SOAP_CUDA(ctx, cudaFuncSetAttribute(k_fir_blists, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const soapgb_activity *act = boxes->act;
        SOAP_TRACED(ctx, "fir_lists",
                    k_fir_blists<<<n_lists, FIR_BLIST_THREADS, smem, ctx->stream>>>(
                        boxes->grid, 2. / boxes->grid, boxes->table, boxes->reg_off, act->t_star, act->t_diff_spot,
                        act->t_diff_fac, solar, va, rank, geo, lcell, ldlt, laux, counts));
        SOAP_LAUNCHED(ctx);
    } else if (bi && gm < (1LL << 24)) {
        // phases: short lists by a per-phase sort of the active cells, the rest by a scan
        int *rank = vb;   // free after the second sort
        SOAP_TRACED(ctx, "fir_rank", k_fir_rank<<<g, 256, 0, ctx->stream>>>(gm, va, rank));
        SOAP_LAUNCHED(ctx);
        SOAP_TRACED(ctx, "fir_lists", k_fir_plists<<<n_lists, 512, 0, ctx->stream>>>(gm, va, rank, geo, temp, bi, solar, lcell, ldlt, laux, counts));
        SOAP_LAUNCHED(ctx);
        SOAP_TRACED(ctx, "fir_lists_scan", k_fir_lists<<<n_lists, 1024, 0, ctx->stream>>>(gm, va, geo, temp, bi, solar, lcell, ldlt, laux, counts, 1));
        SOAP_LAUNCHED(ctx);
    } else {
        SOAP_TRACED(ctx, "fir_lists_scan", k_fir_lists<<<n_lists, 1024, 0, ctx->stream>>>(gm, va, geo, temp, bi, solar, lcell, ldlt, laux, counts, 0));
        SOAP_LAUNCHED(ctx);
    }
    double *pre = (double *)(ws + L.off[FirLayout::PRE]);
    int2 *segs = (int2 *)(ws + L.off[FirLayout::SEGS]);
    int *nseg = (int *)(ws + L.off[FirLayout::NSEG]);
    SOAP_TRACED(ctx, "fir_prefix", k_fir_prefix<<<dim3(n_lists, 2), 256, 0, ctx->stream>>>(gm, counts, lcell, geo, pre, L.pre_stride, L.pre_comp,
                                                            segs, nseg, L.seg_cap, ctx->d_status));
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}

// the tile kernels' arguments for the lists of one workspace
static FirTileArgs make_tile_args(soapgb_ctx *ctx, const FirLayout &L, char *ws, int n, int n_eff, const double *lam,
                                  double los, const FirCubes &fc, long long gm, int solar, int t_norm_fac, void *o0,
                                  void *o1, void *o2, long long out_stride, int n_lists) {
    FirTileArgs A;
    A.n = n;
    A.n_eff = n_eff;
    A.lam = lam;
    A.los = los;
    A.cubes = fc;
    A.list_cell = (const int *)(ws + L.off[FirLayout::LCELL]);
    A.list_dlt = (const double *)(ws + L.off[FirLayout::LDLT]);
    A.counts = (const int *)(ws + L.off[FirLayout::COUNTS]);
    A.pre = (const double *)(ws + L.off[FirLayout::PRE]);
    A.pre_stride = L.pre_stride;
    A.pre_comp = L.pre_comp;
    A.segs = (const int2 *)(ws + L.off[FirLayout::SEGS]);
    A.nseg = (const int *)(ws + L.off[FirLayout::NSEG]);
    A.seg_cap = L.seg_cap;
    A.geo = (const CellGeo *)(ws + L.off[FirLayout::GEO]);
    A.geo32 = (const CellGeo32 *)(ws + L.off[FirLayout::GEO32]);
    A.list_aux = (const double2 *)(ws + L.off[FirLayout::LAUX]);
    A.gm = gm;
    A.solar = solar;
    A.t_norm_fac = t_norm_fac;
    A.out0 = o0;
    A.out1 = o1;
    A.out2 = o2;
    A.out_stride = out_stride;
    A.status = ctx->d_status;
    A.plan = nullptr;
    A.run_list = nullptr;
    A.n_lists_all = n_lists;
    A.wait_limit = ctx->test_wait_limit > 0 ? ctx->test_wait_limit : FIR_WAIT_LIMIT;
    A.drop_plan = (ctx->test_drop_copy == 1) ? 1 : 0;
    A.drop_unit = (ctx->test_drop_copy == 3) ? 1 : 0;
    return A;
}

template <typename T, int MODE, typename OutT>
static int launch_tiles(soapgb_ctx *ctx, const FirLayout &L, char *ws, int n, int n_eff, const double *lam,
                        double los, const FirCubes &fc, long long gm, int solar,
                        int t_norm_fac, void *o0, void *o1, void *o2, long long out_stride, int n_lists,
                        int stage = 7, int l0 = 0, int l1 = -1, const FirPhaseArgs *pa = nullptr) {
    constexpr int NC = (MODE == MODE_QUIET) ? 1 : 4;
    if (l1 < 0) l1 = n_lists;
    FirTileArgs A = make_tile_args(ctx, L, ws, n, n_eff, lam, los, fc, gm, solar, t_norm_fac, o0, o1, o2, out_stride,
                                   n_lists);
    const int ntile = (n + FIR_TILE - 1) / FIR_TILE;
    if constexpr (MODE == MODE_PHASE) {
        // plans of every (phase, tile) (stage 1), then the persistent tile kernel over the
        // phases [l0, l1) (stage 4)
        A.plan = ws + L.off[FirLayout::PLAN];
        // with run / zero lists: only the listed phases are planned and integrated, the
        // others zero-filled; [r0, r1) and [z0, z1) are the parts of the lists in [l0, l1)
        const bool lists = pa && pa->run_list;
        int r0 = l0, r1 = l1, z0 = 0, z1 = 0;
        if (lists) {
            A.run_list = pa->run_list;
            r0 = (int)(std::lower_bound(pa->run_host, pa->run_host + pa->n_run, l0) - pa->run_host);
            r1 = (int)(std::lower_bound(pa->run_host, pa->run_host + pa->n_run, l1) - pa->run_host);
            z0 = (int)(std::lower_bound(pa->zero_host, pa->zero_host + pa->n_zero, l0) - pa->zero_host);
            z1 = (int)(std::lower_bound(pa->zero_host, pa->zero_host + pa->n_zero, l1) - pa->zero_host);
        }
        const int n_plan = lists ? pa->n_run : n_lists;
        if ((stage & 1) && n_plan > 0) {
            size_t smem_p = ((sizeof(FirPrePlan<T>) + 15) & ~size_t(15)) + sizeof(FirSeg) * 2 * (size_t)L.seg_cap;
            SOAP_CUDA(ctx, cudaFuncSetAttribute(k_fir_plan<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_p));
            SOAP_TRACED(ctx, "fir_plan",
                        k_fir_plan<T><<<dim3(ntile, n_plan), FIR_PLAN_THREADS, smem_p, ctx->stream>>>(A));
            SOAP_LAUNCHED(ctx);
        }
        if ((stage & 4) && z1 > z0 && pa->zero_fill) {
            SOAP_TRACED(ctx, "fir_zero",
                        k_fir_zero<T><<<dim3((n + 255) / 256, z1 - z0), 256, 0, ctx->stream>>>(
                            n, pa->zero_list + z0, (T *)o0, (T *)o1, (T *)o2, out_stride));
            SOAP_LAUNCHED(ctx);
        }
        if ((stage & 4) && r1 > r0) {
            const int nrun = ntile * (r1 - r0);
            size_t smem_t = fir_pp_smem_fixed<T>() + sizeof(FirSeg) * 2 * (size_t)L.seg_cap;
            auto kern = ctx->fir_compensated ? k_fir_pp<T, true, false> : k_fir_pp<T, false, false>;
            SOAP_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_t));
            int per_sm = 0;
            SOAP_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, FIR_THREADS, smem_t));
            const int nblk = std::max(1, std::min(nrun, std::max(per_sm, 1) * std::max(ctx->num_sms, 1)));
            SOAP_TRACED(ctx, "fir_tile_phase",
                        kern<<<nblk, FIR_THREADS, smem_t, ctx->stream>>>(A, ntile, r0, r1 - r0, ntile * n_lists,
                                                                         nullptr, nullptr, 0));
            SOAP_LAUNCHED(ctx);
        }
        return SOAPGB_OK;
    }
    size_t smem = fir_smem_fixed<T, NC>() + sizeof(FirSeg) * (size_t)(MODE == MODE_PHASE ? 2 : 1) * L.seg_cap;
    SOAP_CUDA(ctx, cudaFuncSetAttribute(k_fir<T, MODE, OutT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // tiles cover [0, n): tiles past n_eff only write the zero tail
    dim3 g((n + FIR_TILE - 1) / FIR_TILE, n_lists);
    SOAP_TRACED(ctx, MODE == MODE_QUIET ? "fir_tile_quiet" : "fir_tile_phase", k_fir<T, MODE, OutT><<<g, FIR_THREADS, smem, ctx->stream>>>(A));
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}

int fir_quiet(soapgb_ctx *ctx, int form, const FirQuietArgs &a, char *scratch, const FirPlanSizes &plan) {
    (void)plan;
    if (a.n_mu > FIR_MAX_MU)
        return set_error(ctx, SOAPGB_ERR_ARG, "collapsed forms support at most %d mu bins (got %d)", FIR_MAX_MU, a.n_mu);
    const long long gm = a.gm;
    FirLayout L = fir_layout(form, a.n, a.n_mu, gm, 1, 1);
    char *ws = scratch;
    CellGeo *geo = (CellGeo *)(ws + L.off[FirLayout::GEO]);
    CellGeo32 *geo32 = (CellGeo32 *)(ws + L.off[FirLayout::GEO32]);
    double lambda0 = a.lambda0;
    int rc = fir_prepare(ctx, a.wave, a.n_eff, a.step, gm, a.delta, a.limb, nullptr, a.region, a.n_mu, geo, geo32,
                         &lambda0);
    if (rc) return rc;
    rc = fir_lists(ctx, L, ws, gm, 1, nullptr, nullptr, 0);
    if (rc) return rc;
    size_t cube_elems = (size_t)a.n * a.n_mu;
    void *cube = ws + L.off[FirLayout::CUBE0];
    FirCubes fc{};
    fc.c[0] = cube;
    const double los = lambda0 / a.step;
    // one cube, or two over the same lists (the typed copy is rewritten in stream order)
    for (int q = 0; q < (a.cube2 ? 2 : 1); ++q) {
        const double *src = q ? a.cube2 : a.cube;
        double *out = q ? a.out2 : a.out;
        if (form == SOAPGB_FAST32) {
            SOAP_TRACED(ctx, "cube_types", k_to_type<float><<<grid_for(ctx, cube_elems, 256), 256, 0, ctx->stream>>>(cube_elems, src, nullptr, (float *)cube));
            SOAP_LAUNCHED(ctx);
            rc = launch_tiles<float, MODE_QUIET, double>(ctx, L, ws, a.n, a.n_eff, a.wave, los, fc, gm, 0, 0, out,
                                                         nullptr, nullptr, 0, 1);
        } else {
            SOAP_TRACED(ctx, "cube_types", k_to_type<double><<<grid_for(ctx, cube_elems, 256), 256, 0, ctx->stream>>>(cube_elems, src, nullptr, (double *)cube));
            SOAP_LAUNCHED(ctx);
            rc = launch_tiles<double, MODE_QUIET, double>(ctx, L, ws, a.n, a.n_eff, a.wave, los, fc, gm, 0, 0, out,
                                                          nullptr, nullptr, 0, 1);
        }
        if (rc) return rc;
    }
    return SOAPGB_OK;
}

// the typed cubes a phase integration reads: its workspace slots, or the shared copies
static FirCubes phase_cubes(const FirLayout &L, char *ws, const FirPhaseArgs &a) {
    FirCubes fc{};
    if (a.typed) {
        for (int q = 0; q < 6; ++q) fc.c[q] = a.typed->c[q];
        fc.spot_sed2 = (const float2 *)a.typed->spot_sed2;
        fc.fac_sed2 = (const float2 *)a.typed->fac_sed2;
    } else {
        for (int q = 0; q < 6; ++q) fc.c[q] = ws + L.off[FirLayout::CUBE0 + q];
        fc.spot_sed2 = (const float2 *)(ws + L.off[FirLayout::SED2A]);
        fc.fac_sed2 = (const float2 *)(ws + L.off[FirLayout::SED2B]);
    }
    fc.spot_sed = a.cubes->spot_sed;
    fc.fac_sed = a.cubes->fac_sed;
    return fc;
}

int fir_phase(soapgb_ctx *ctx, int form, const FirPhaseArgs &a, char *scratch, const FirPlanSizes &plan) {
    (void)plan;
    const int n_mu = a.cubes->n_mu;
    if (n_mu > FIR_MAX_MU)
        return set_error(ctx, SOAPGB_ERR_ARG, "collapsed forms support at most %d mu bins (got %d)", FIR_MAX_MU, n_mu);
    if ((form == SOAPGB_FAST32) != (a.out_f32 != 0))
        return set_error(ctx, SOAPGB_ERR_ARG, "FP32 deficits go with the FP32 form only");
    FirLayout L = fir_layout(form, a.n, n_mu, a.gm, 6, a.n_phase, a.typed != nullptr);
    char *ws = scratch;
    CellGeo *geo = (CellGeo *)(ws + L.off[FirLayout::GEO]);
    CellGeo32 *geo32 = (CellGeo32 *)(ws + L.off[FirLayout::GEO32]);
    double lambda0 = a.lambda0;
    if (a.stage & FIR_STAGE_GEOMETRY) {
        int rc = fir_prepare(ctx, a.wave, a.n_eff, a.step, a.gm, a.delta, a.limb, a.lb, a.region, n_mu, geo, geo32,
                             &lambda0);
        if (rc) return rc;
        if (!a.bi && !a.table) return set_error(ctx, SOAPGB_ERR_ARG, "fir_phase: neither maps nor a region table");
        rc = fir_lists(ctx, L, ws, a.gm, a.n_phase, a.temp, a.bi, a.act->solar, a.bi ? nullptr : &a);
        if (rc) return rc;
    } else if (!(lambda0 > 0.0)) {
        return set_error(ctx, SOAPGB_ERR_ARG, "fir_phase: the run stage alone needs lambda0");
    }
    const soapgb_cubes &c = *a.cubes;
    FirCubes fc = phase_cubes(L, ws, a);
    if (a.stage & FIR_STAGE_CUBES) {
        if (a.typed) return set_error(ctx, SOAPGB_ERR_ARG, "fir_phase: shared typed cubes are made by fir_typed_cubes");
        void *d[2] = {const_cast<void *>(fc.c[0]), const_cast<void *>(fc.c[1])};
        int rc = typed_cubes_into(ctx, form, a.n, c, d, (float2 *)fc.spot_sed2, (float2 *)fc.fac_sed2);
        if (rc) return rc;
    }
    const int t_norm_fac = (int)(a.act->t_star + a.act->t_diff_fac + 0.9 - 216.8);
    const double los = lambda0 / a.step;
    const int st = (a.stage & FIR_STAGE_GEOMETRY ? 1 : 0) | (a.stage & FIR_STAGE_RUN ? 4 : 0);
    const int l1 = (a.l1 < 0) ? a.n_phase : a.l1;
    if (form == SOAPGB_FAST32)
        return launch_tiles<float, MODE_PHASE, float>(ctx, L, ws, a.n, a.n_eff, a.wave, los, fc, a.gm,
                                                      a.act->solar, t_norm_fac, a.flux, a.bconv, a.tot, a.out_stride,
                                                      a.n_phase, st, a.l0, l1, &a);
    return launch_tiles<double, MODE_PHASE, double>(ctx, L, ws, a.n, a.n_eff, a.wave, los, fc, a.gm,
                                                    a.act->solar, t_norm_fac, a.flux, a.bconv, a.tot, a.out_stride,
                                                    a.n_phase, st, a.l0, l1, &a);
}

size_t fir_tile_args_bytes() { return sizeof(FirTileArgs); }

int fir_phase_star_args(soapgb_ctx *ctx, int form, const FirPhaseArgs &a, char *scratch, void *out) {
    if (form != SOAPGB_FAST32) return set_error(ctx, SOAPGB_ERR_ARG, "several stars in one launch: FP32 form only");
    if (!a.typed || !(a.lambda0 > 0.0) || !a.run_list)
        return set_error(ctx, SOAPGB_ERR_ARG, "fir_phase_star_args: needs shared typed cubes, lambda0 and run lists");
    const int n_mu = a.cubes->n_mu;
    FirLayout L = fir_layout(form, a.n, n_mu, a.gm, 6, a.n_phase, true);
    char *ws = scratch;
    const int t_norm_fac = (int)(a.act->t_star + a.act->t_diff_fac + 0.9 - 216.8);
    FirTileArgs A = make_tile_args(ctx, L, ws, a.n, a.n_eff, a.wave, a.lambda0 / a.step, phase_cubes(L, ws, a), a.gm,
                                   a.act->solar, t_norm_fac, a.flux, a.bconv, a.tot, a.out_stride, a.n_phase);
    A.plan = ws + L.off[FirLayout::PLAN];
    A.run_list = a.run_list;
    memcpy(out, &A, sizeof(A));
    return SOAPGB_OK;
}

int fir_phase_multi(soapgb_ctx *ctx, int form, const void *star0_args, const void *d_star_args, const int2 *d_items,
                    int n_items, int chunk, int blocks_per_sm) {
    if (form != SOAPGB_FAST32) return set_error(ctx, SOAPGB_ERR_ARG, "several stars in one launch: FP32 form only");
    if (n_items <= 0) return SOAPGB_OK;
    FirTileArgs A0;
    memcpy(&A0, star0_args, sizeof(A0));
    const int ntile = (A0.n + FIR_TILE - 1) / FIR_TILE;
    // every star's segments fit the capacity of the cubes' mu bins (seg_cap = 2 n_mu)
    size_t smem_t = fir_pp_smem_fixed<float>() + sizeof(FirSeg) * 2 * (size_t)A0.seg_cap;
    auto kern = ctx->fir_compensated ? k_fir_pp<float, true, true> : k_fir_pp<float, false, true>;
    SOAP_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_t));
    int per_sm = 0;
    SOAP_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, FIR_THREADS, smem_t));
    per_sm = std::max(per_sm, 1);
    if (blocks_per_sm > 0) per_sm = std::min(per_sm, blocks_per_sm);
    const long long total = (long long)n_items * ntile;
    if (total >= (1LL << 31)) return set_error(ctx, SOAPGB_ERR_ARG, "too many (phase, tile) pairs in one launch");
    const int nblk = (int)std::max(1LL, std::min(total, (long long)per_sm * std::max(ctx->num_sms, 1)));
    SOAP_TRACED(ctx, "fir_tile_phase_multi",
                kern<<<nblk, FIR_THREADS, smem_t, ctx->stream>>>(A0, ntile, 0, n_items, 0,
                                                                 (const FirTileArgs *)d_star_args, d_items, chunk));
    SOAP_LAUNCHED(ctx);
    return SOAPGB_OK;
}