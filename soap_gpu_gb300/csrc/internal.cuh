// Internal declarations shared by the libsoapgb translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/soapgb.h"

#define SOAP_C_LIGHT 299792458.
#define SOAP_PI 3.141592653589793238463

// one traced launch: events recorded around it on the context's stream
struct SoapTraceSpan {
    const char *name;
    cudaEvent_t a, b;
};

struct soapgb_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;      // stream in use
    cudaStream_t own_stream = nullptr;  // stream created by the context
    std::string err;
    // device workspace (grown on demand, reused across calls)
    char *ws = nullptr;
    size_t ws_size = 0;
    // device status word written by kernels (0 = ok)
    int *d_status = nullptr;
    long long launches = 0;
    int num_sms = 0;
    // second stream for copies that overlap kernels (created on first use) and events
    cudaStream_t copy_stream = nullptr;
    cudaStream_t d2h_stream = nullptr;   // device-to-host copies beside the copy stream's uploads
    std::vector<cudaEvent_t> sync_events;
    // second compute stream for independent stages (created on first use) and its
    // ordering events: main -> aux at the start, aux -> main at the join, and a second
    // aux -> main point where the main stream needs only the first part of the aux work
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t aux_events[3] = {nullptr, nullptr, nullptr};
    // stream of the highest priority for latency-bound stages on the critical path (the
    // block scheduler dispatches its pending blocks first) and its join event
    cudaStream_t geo_stream = nullptr;
    cudaEvent_t geo_event = nullptr;
    // a second aux stream (independent set-up work beside the first, dispatched ahead of
    // it at the highest priority) and its join event
    cudaStream_t aux2_stream = nullptr;
    cudaEvent_t aux2_event = nullptr;
    // recorded on the previous stream when soapgb_set_stream switches streams: work the
    // context queued there (which may still use its scratch) precedes the new stream's
    cudaEvent_t switch_event = nullptr;
    // wave[0], wave[1], wave[n_eff - 1] of the last device wavelength array seen (read
    // once; later calls with the same array confirm them on the device, status 51)
    const double *edge_wave = nullptr;
    int edge_n = 0, edge_n_eff = 0;
    double edge_w3[3] = {0.0, 0.0, 0.0};
    // FP32 per-phase integration: compensated (Kahan) output sums (soapgb_set_compensated)
    bool fir_compensated = true;
    // failure-path tests only, read from the environment at context creation:
    // SOAPGB_TEST_WAIT_LIMIT polls per bounded wait of the staged-copy kernels (0: the
    // default 2^24) and SOAPGB_TEST_DROP_COPY, a staged copy whose bytes are expected but
    // never issued, so that its wait runs out (1: the integration kernel's first plan
    // copy, status 41; 2: the FP32 convolution's first window, status 42; 3: the
    // integration kernel's first window copy of each block, status 41)
    long long test_wait_limit = 0;
    int test_drop_copy = 0;
    // per-kernel tracing (soapgb_trace_enable): spans recorded since the last report
    bool trace = false;
    std::vector<SoapTraceSpan> spans;
    std::vector<cudaEvent_t> ev_free;
};

namespace soapgb {

int set_error(soapgb_ctx *ctx, int code, const char *fmt, ...);
int cuda_check(soapgb_ctx *ctx, cudaError_t e, const char *what);
#define SOAP_CUDA(ctx, call)                                         \
    do {                                                             \
        cudaError_t _e = (call);                                     \
        if (_e != cudaSuccess) return soapgb::cuda_check(ctx, _e, #call); \
    } while (0)
#define SOAP_LAUNCHED(ctx)                                                   \
    do {                                                                     \
        (ctx)->launches++;                                                   \
        cudaError_t _e = cudaGetLastError();                                 \
        if (_e != cudaSuccess) return soapgb::cuda_check(ctx, _e, "kernel launch"); \
    } while (0)

// Makes a context's device current for the duration of an entry point and gives the
// caller's current device back when the entry point returns, so no call changes the
// calling thread's device as a side effect.
struct DeviceGuard {
    int prev = -1;
    bool changed = false;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            cudaGetLastError();
            prev = -1;
        }
        if (prev != device) {
            err = cudaSetDevice(device);
            changed = (err == cudaSuccess && prev >= 0);
        }
    }
    ~DeviceGuard() {
        if (changed) cudaSetDevice(prev);
    }
    DeviceGuard(const DeviceGuard &) = delete;
    DeviceGuard &operator=(const DeviceGuard &) = delete;
};
#define SOAP_DEVICE(ctx)                                                              \
    soapgb::DeviceGuard _soap_device_guard((ctx)->device);                           \
    if (_soap_device_guard.err != cudaSuccess)                                        \
        return soapgb::cuda_check(ctx, _soap_device_guard.err, "cudaSetDevice")

// Bump allocator over the context workspace.  Usage: plan sizes with add(),
// then commit() (grows the workspace if needed), then take pointers with get().
struct Workspace {
    soapgb_ctx *ctx;
    std::vector<size_t> sizes;
    std::vector<size_t> offs;
    size_t total = 0;
    explicit Workspace(soapgb_ctx *c) : ctx(c) {}
    int add(size_t bytes) {
        size_t off = (total + 255) & ~size_t(255);
        offs.push_back(off);
        sizes.push_back(bytes);
        total = off + bytes;
        return (int)offs.size() - 1;
    }
    int commit();
    template <class T> T *get(int slot) const { return reinterpret_cast<T *>(ctx->ws + offs[slot]); }
};

// Copy an input array into the workspace when it is a host array; returns the
// device pointer to use.  `slot` must have been planned with add(bytes) when mem
// is host (pass slot -1 for device mode).
const void *stage_in(soapgb_ctx *ctx, int mem, const void *p, size_t bytes, void *dst, int *rc);

int check_status(soapgb_ctx *ctx, const char *what);
// device status word: a cached wavelength edge value no longer matches the array
constexpr int SOAPGB_ST_EDGES = 51;
constexpr int SOAPGB_ST_FIT_SINGULAR = 61;   // the fit adjoint met a singular 4x4 system
// true for memory the host can read directly (pageable or page-locked host memory)
bool host_readable(const void *p);
// copy a small descriptor array to the host: directly from host memory, or from device
// memory with a synchronisation of the context's stream
int read_descriptor(soapgb_ctx *ctx, void *dst, const void *src, size_t bytes);
// w3 = (wave[0], wave[1], wave[n_eff - 1]) without a synchronisation when the same
// device array was seen before (a one-thread kernel confirms the values on the device)
int wave_edges(soapgb_ctx *ctx, int mem, const double *wave, int n, int n_eff, double *w3);

// number of visible cells etc. via ordered compaction helpers (regions.cu)
int compact_cells(soapgb_ctx *ctx, int n_lists, int cells_per_list, const double *key,
                  double lo, double hi, int key_stride, int *idx_out, int *count_out);

int grid_for(soapgb_ctx *ctx, long long work, int block);

// the context's copy stream and at least `count` synchronisation events (created once)
int copy_resources(soapgb_ctx *ctx, int count);
int aux_resources(soapgb_ctx *ctx);

// Launches made while an AuxScope is alive go to the context's aux stream (the stream
// member is switched and restored; every launch of the library reads ctx->stream).
struct AuxScope {
    soapgb_ctx *ctx;
    cudaStream_t saved;
    explicit AuxScope(soapgb_ctx *c) : ctx(c), saved(c->stream) { ctx->stream = ctx->aux_stream; }
    AuxScope(soapgb_ctx *c, cudaStream_t s) : ctx(c), saved(c->stream) { ctx->stream = s; }
    ~AuxScope() { ctx->stream = saved; }
};

// Scope around a kernel launch: with tracing on, CUDA events on the context's stream
// bracket the launch (records nothing otherwise).
struct TraceScope {
    soapgb_ctx *ctx;
    const char *name;
    cudaStream_t stream;
    cudaEvent_t a = nullptr;
    TraceScope(soapgb_ctx *c, const char *n);                    // on the context's stream
    TraceScope(soapgb_ctx *c, const char *n, cudaStream_t s);    // on stream s (copies)
    ~TraceScope();
};

}  // namespace soapgb

// a kernel launch bracketed by trace events (the launch statement may contain commas)
#define SOAP_TRACED(ctx, name, ...)                  \
    do {                                             \
        soapgb::TraceScope _soap_ts((ctx), (name)); \
        __VA_ARGS__;                                 \
    } while (0)

// ---------------------------------------------------------------------------
// Device helpers: the reference's expressions, written out once.
// ---------------------------------------------------------------------------

// float -> double by bit manipulation on the integer pipes (GB300's FP64 pipe runs at
// 1/64 of the FP32 rate; this keeps FP32 results' exact value in FP64 storage)
__device__ __forceinline__ double soap_f32_to_f64(float f) {
    unsigned b = __float_as_uint(f);
    unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
    unsigned e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
    unsigned long long r;
    if (e == 0u) {
        if (m != 0u) return (double)f;   // subnormal: rare, convert on the FP64 pipe
        r = sign;
    } else if (e == 255u) {
        r = sign | 0x7ff0000000000000ULL | ((unsigned long long)m << 29);
    } else {
        r = sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
    }
    return __longlong_as_double((long long)r);
}

// order-preserving map of a double onto uint64 (integer compares and atomics)
__device__ __forceinline__ unsigned long long soap_ord64(double v) {
    unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return (u & 0x8000000000000000ULL) ? ~u : (u | 0x8000000000000000ULL);
}

// Packed FP32 pairs (the f32x2 instructions of the sm_100 family): one instruction
// does two FP32 operations with the rounding of each done separately.
__device__ __forceinline__ void soap_add2(float &x, float &y, float a, float b) {   // (x, y) += (a, b)
    asm("{\n\t.reg .b64 p, q;\n\tmov.b64 p, {%0, %1};\n\tmov.b64 q, {%2, %3};\n\t"
        "add.rn.f32x2 p, p, q;\n\tmov.b64 {%0, %1}, p;\n\t}"
        : "+f"(x), "+f"(y)
        : "f"(a), "f"(b));
}
__device__ __forceinline__ void soap_sub2(float &x, float &y, float a, float b) {   // (x, y) -= (a, b)
    asm("{\n\t.reg .b64 p, q;\n\tmov.b64 p, {%0, %1};\n\tmov.b64 q, {%2, %3};\n\t"
        "sub.rn.f32x2 p, p, q;\n\tmov.b64 {%0, %1}, p;\n\t}"
        : "+f"(x), "+f"(y)
        : "f"(a), "f"(b));
}
__device__ __forceinline__ void soap_mul2(float &x, float &y, float a, float b, float c, float d) {   // (a c, b d)
    asm("{\n\t.reg .b64 p, q, r;\n\tmov.b64 p, {%2, %3};\n\tmov.b64 q, {%4, %5};\n\t"
        "mul.rn.f32x2 r, p, q;\n\tmov.b64 {%0, %1}, r;\n\t}"
        : "=f"(x), "=f"(y)
        : "f"(a), "f"(b), "f"(c), "f"(d));
}
// (x, y) = (a, b) * (c, d) + (x, y)
__device__ __forceinline__ void soap_fma2(float &x, float &y, float a, float b, float c, float d) {
    asm("{\n\t.reg .b64 p, q, r;\n\tmov.b64 p, {%2, %3};\n\tmov.b64 q, {%4, %5};\n\tmov.b64 r, {%0, %1};\n\t"
        "fma.rn.f32x2 r, p, q, r;\n\tmov.b64 {%0, %1}, r;\n\t}"
        : "+f"(x), "+f"(y)
        : "f"(a), "f"(b), "f"(c), "f"(d));
}

// Delta_lambda, SOAP_initialize.cu:55-66
__device__ __forceinline__ double soap_delta_lambda(double line_width, double lambda_line0) {
    double beta = line_width / SOAP_C_LIGHT;
    return -1 * lambda_line0 * (1 - sqrt((1 + beta) / (1 - beta)));
}

// Per-cell Doppler constants of fast_shift / fast_interp_new (SOAP_initialize.cu:117-167).
struct CellShift {
    double fbeta;     // sqrt((1+b)/(1-b)) - 1
    double sq;        // sqrt((1+b)/(1-b))
    double off;       // fbeta * lambda0 / step
};

__device__ __forceinline__ CellShift soap_cell_shift(double delta, double lambda0, double step) {
    CellShift c;
    double beta = delta * 1000. / SOAP_C_LIGHT;
    c.sq = sqrt((1 + beta) / (1 - beta));
    c.fbeta = -1 * (1 - c.sq);
    c.off = __ddiv_rn(__dmul_rn(c.fbeta, lambda0), step);
    return c;
}

// ceil of the shifted source position x_i = i (1 + fbeta) + fbeta lambda0 / step,
// evaluated without contraction (one rounding per operation, as the oracle does).
__device__ __forceinline__ long long soap_ceil_pos(long long i, const CellShift &c) {
    double x = __dadd_rn(__dmul_rn((double)i, 1 + c.fbeta), c.off);
    return (long long)ceil(x);
}

// shifted wavelength lambda'_i = lambda_i + Delta_lambda(v, lambda_i)
__device__ __forceinline__ double soap_lshift(double lam, const CellShift &c) {
    return lam + (-1 * lam * (1 - c.sq));
}

// Owner of output pixel j: the source i in [0, n_eff-2] with
// ceil(x_i) <= j < ceil(x_{i+1}); returns -1 if none.
__device__ __forceinline__ long long soap_owner(long long j, int n_eff, const CellShift &c) {
    // seed: x = (j - off) / (1 + f) to second order in f; the two loops below then pin
    // the owner exactly, so the seed's rounding never reaches the result
    const double x = (double)j - c.off;
    long long i = (long long)floor(x * (1.0 - c.fbeta + c.fbeta * c.fbeta));
    if (i < -1) i = -1;
    if (i > n_eff - 1) i = n_eff - 1;
    // advance while the next source still starts at or before j
    while (i + 1 <= n_eff - 1 && soap_ceil_pos(i + 1, c) <= j) ++i;
    // retreat while this source starts after j
    while (i >= 0 && soap_ceil_pos(i, c) > j) --i;
    if (i < 0 || i > n_eff - 2) return -1;
    return i;
}
