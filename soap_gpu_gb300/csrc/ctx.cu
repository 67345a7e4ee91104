// Context, error reporting and device workspace of libsoapgb.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <algorithm>

#include "internal.cuh"

namespace soapgb {

int set_error(soapgb_ctx *ctx, int code, const char *fmt, ...) {
    if (ctx) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return code;
}

int cuda_check(soapgb_ctx *ctx, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return SOAPGB_OK;
    int code = (e == cudaErrorMemoryAllocation) ? SOAPGB_ERR_ALLOC : SOAPGB_ERR_CUDA;
    return set_error(ctx, code, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

int Workspace::commit() {
    if (total <= ctx->ws_size) return SOAPGB_OK;
    // grow: wait for in-flight work that may still read the old buffer
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, "workspace sync");
    if (ctx->ws) cudaFree(ctx->ws);
    ctx->ws = nullptr;
    ctx->ws_size = 0;
    size_t want = total + (total >> 3);  // 12.5% headroom for the next call
    e = cudaMalloc((void **)&ctx->ws, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        e = cudaMalloc((void **)&ctx->ws, total);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error(ctx, SOAPGB_ERR_ALLOC, "workspace allocation of %zu bytes failed", total);
        }
        want = total;
    }
    ctx->ws_size = want;
    return SOAPGB_OK;
}

const void *stage_in(soapgb_ctx *ctx, int mem, const void *p, size_t bytes, void *dst, int *rc) {
    *rc = SOAPGB_OK;
    if (mem == SOAPGB_DEVICE || p == nullptr || bytes == 0) return p;
    cudaError_t e = cudaMemcpyAsync(dst, p, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) {
        *rc = cuda_check(ctx, e, "host to device copy");
        return nullptr;
    }
    return dst;
}

int check_status(soapgb_ctx *ctx, const char *what) {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, what);
    if (h != 0) {
        cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream);
        if (h == SOAPGB_ST_EDGES) {
            ctx->edge_wave = nullptr;
            return set_error(ctx, SOAPGB_ERR_DEVICE,
                             "%s: device status %d: the wavelength array changed after an earlier call read its "
                             "first, second or last value; the calls since then used the old values",
                             what, h);
        }
        return set_error(ctx, SOAPGB_ERR_DEVICE, "%s: device status %d", what, h);
    }
    return SOAPGB_OK;
}

bool host_readable(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return true;   // not known to CUDA: ordinary host memory
    }
    return at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeUnregistered;
}

int read_descriptor(soapgb_ctx *ctx, void *dst, const void *src, size_t bytes) {
    if (bytes == 0) return SOAPGB_OK;
    if (host_readable(src)) {
        memcpy(dst, src, bytes);
        return SOAPGB_OK;
    }
    SOAP_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SOAPGB_OK;
}

__global__ void k_check_edges(const double *__restrict__ wave, int n_eff, double w0, double w1, double wl,
                              int *status) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const bool same = __double_as_longlong(wave[0]) == __double_as_longlong(w0) &&
                      __double_as_longlong(wave[1]) == __double_as_longlong(w1) &&
                      __double_as_longlong(wave[n_eff - 1]) == __double_as_longlong(wl);
    if (!same) atomicExch(status, SOAPGB_ST_EDGES);
}

int wave_edges(soapgb_ctx *ctx, int mem, const double *wave, int n, int n_eff, double *w3) {
    if (mem == SOAPGB_HOST || host_readable(wave)) {
        w3[0] = wave[0];
        w3[1] = wave[1];
        w3[2] = wave[n_eff - 1];
        return SOAPGB_OK;
    }
    if (ctx->edge_wave == wave && ctx->edge_n == n && ctx->edge_n_eff == n_eff) {
        w3[0] = ctx->edge_w3[0];
        w3[1] = ctx->edge_w3[1];
        w3[2] = ctx->edge_w3[2];
        k_check_edges<<<1, 32, 0, ctx->stream>>>(wave, n_eff, w3[0], w3[1], w3[2], ctx->d_status);
        SOAP_LAUNCHED(ctx);
        return SOAPGB_OK;
    }
    SOAP_CUDA(ctx, cudaMemcpyAsync(w3, wave, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SOAP_CUDA(ctx, cudaMemcpyAsync(w3 + 2, wave + n_eff - 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->edge_wave = wave;
    ctx->edge_n = n;
    ctx->edge_n_eff = n_eff;
    for (int q = 0; q < 3; ++q) ctx->edge_w3[q] = w3[q];
    return SOAPGB_OK;
}

static cudaEvent_t trace_event(soapgb_ctx *ctx) {
    if (!ctx->ev_free.empty()) {
        cudaEvent_t e = ctx->ev_free.back();
        ctx->ev_free.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

TraceScope::TraceScope(soapgb_ctx *c, const char *n) : TraceScope(c, n, c ? c->stream : nullptr) {}

TraceScope::TraceScope(soapgb_ctx *c, const char *n, cudaStream_t s) : ctx(c), name(n), stream(s) {
    if (!ctx || !ctx->trace) return;
    a = trace_event(ctx);
    if (a) cudaEventRecord(a, stream);
}

TraceScope::~TraceScope() {
    if (!a) return;
    cudaEvent_t b = trace_event(ctx);
    if (!b) {
        ctx->ev_free.push_back(a);
        return;
    }
    cudaEventRecord(b, stream);
    ctx->spans.push_back(SoapTraceSpan{name, a, b});
}

int aux_resources(soapgb_ctx *ctx) {
    if (!ctx->aux_stream) SOAP_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking));
    for (int q = 0; q < 3; ++q)
        if (!ctx->aux_events[q]) SOAP_CUDA(ctx, cudaEventCreateWithFlags(&ctx->aux_events[q], cudaEventDisableTiming));
    int least = 0, greatest = 0;
    SOAP_CUDA(ctx, cudaDeviceGetStreamPriorityRange(&least, &greatest));
    if (!ctx->geo_stream)
        SOAP_CUDA(ctx, cudaStreamCreateWithPriority(&ctx->geo_stream, cudaStreamNonBlocking, greatest));
    if (!ctx->geo_event) SOAP_CUDA(ctx, cudaEventCreateWithFlags(&ctx->geo_event, cudaEventDisableTiming));
    if (!ctx->aux2_stream)
        SOAP_CUDA(ctx, cudaStreamCreateWithPriority(&ctx->aux2_stream, cudaStreamNonBlocking, greatest));
    if (!ctx->aux2_event) SOAP_CUDA(ctx, cudaEventCreateWithFlags(&ctx->aux2_event, cudaEventDisableTiming));
    return SOAPGB_OK;
}

int copy_resources(soapgb_ctx *ctx, int count) {
    if (!ctx->copy_stream) SOAP_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    if (!ctx->d2h_stream) SOAP_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->d2h_stream, cudaStreamNonBlocking));
    while ((int)ctx->sync_events.size() < count) {
        cudaEvent_t e = nullptr;
        SOAP_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->sync_events.push_back(e);
    }
    return SOAPGB_OK;
}

int grid_for(soapgb_ctx *ctx, long long work, int block) {
    long long g = (work + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 0x7fffffffLL) g = 0x7fffffffLL;
    (void)ctx;
    return (int)g;
}

}  // namespace soapgb

using namespace soapgb;

extern "C" {

const char *soapgb_version(void) { return "soapgb 0.1 (sm_103a)"; }

int soapgb_ctx_create(int device, soapgb_ctx **out) {
    if (!out) return SOAPGB_ERR_ARG;
    *out = nullptr;
    soapgb_ctx *ctx = new soapgb_ctx();
    ctx->device = device;
    soapgb::DeviceGuard guard(device);
    cudaError_t e = guard.err;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_status, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) {
        int rc = cuda_check(ctx, e, "soapgb_ctx_create");
        // keep the context so the caller can read the message, but mark it unusable
        ctx->stream = nullptr;
        *out = ctx;
        return rc;
    }
    ctx->stream = ctx->own_stream;
    if (const char *v = getenv("SOAPGB_TEST_WAIT_LIMIT")) ctx->test_wait_limit = std::max(0LL, atoll(v));
    if (const char *v = getenv("SOAPGB_TEST_DROP_COPY")) ctx->test_drop_copy = atoi(v);
    *out = ctx;
    return SOAPGB_OK;
}

int soapgb_trace_enable(soapgb_ctx *ctx, int on) {
    if (!ctx) return SOAPGB_ERR_ARG;
    for (auto &sp : ctx->spans) {
        ctx->ev_free.push_back(sp.a);
        ctx->ev_free.push_back(sp.b);
    }
    ctx->spans.clear();
    ctx->trace = (on != 0);
    return SOAPGB_OK;
}

int soapgb_trace_report(soapgb_ctx *ctx, char *buf, size_t len) {
    if (!ctx || !buf || len == 0) return SOAPGB_ERR_ARG;
    SOAP_DEVICE(ctx);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, "soapgb_trace_report");
    // aggregate by name, in first-seen order
    std::vector<const char *> names;
    std::vector<int> counts;
    std::vector<double> ms;
    for (auto &sp : ctx->spans) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, sp.a, sp.b) != cudaSuccess) {
            cudaGetLastError();
            t = 0.f;
        }
        size_t k = 0;
        while (k < names.size() && strcmp(names[k], sp.name) != 0) ++k;
        if (k == names.size()) {
            names.push_back(sp.name);
            counts.push_back(0);
            ms.push_back(0.0);
        }
        counts[k] += 1;
        ms[k] += t;
        ctx->ev_free.push_back(sp.a);
        ctx->ev_free.push_back(sp.b);
    }
    ctx->spans.clear();
    size_t used = 0;
    buf[0] = '\0';
    for (size_t k = 0; k < names.size(); ++k) {
        int w = snprintf(buf + used, len - used, "%s %d %.6f\n", names[k], counts[k], ms[k]);
        if (w < 0 || (size_t)w >= len - used) return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_trace_report: buffer too small");
        used += (size_t)w;
    }
    return SOAPGB_OK;
}

int soapgb_ctx_destroy(soapgb_ctx *ctx) {
    if (!ctx) return SOAPGB_OK;
    {
    soapgb::DeviceGuard guard(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto &sp : ctx->spans) {
        cudaEventDestroy(sp.a);
        cudaEventDestroy(sp.b);
    }
    for (auto e : ctx->ev_free) cudaEventDestroy(e);
    for (auto e : ctx->sync_events) cudaEventDestroy(e);
    for (auto e : ctx->aux_events)
        if (e) cudaEventDestroy(e);
    if (ctx->aux_stream) {
        cudaStreamSynchronize(ctx->aux_stream);
        cudaStreamDestroy(ctx->aux_stream);
    }
    if (ctx->geo_event) cudaEventDestroy(ctx->geo_event);
    if (ctx->switch_event) cudaEventDestroy(ctx->switch_event);
    if (ctx->aux2_event) cudaEventDestroy(ctx->aux2_event);
    if (ctx->aux2_stream) {
        cudaStreamSynchronize(ctx->aux2_stream);
        cudaStreamDestroy(ctx->aux2_stream);
    }
    if (ctx->geo_stream) {
        cudaStreamSynchronize(ctx->geo_stream);
        cudaStreamDestroy(ctx->geo_stream);
    }
    if (ctx->d2h_stream) {
        cudaStreamSynchronize(ctx->d2h_stream);
        cudaStreamDestroy(ctx->d2h_stream);
    }
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
    }
    if (ctx->ws) cudaFree(ctx->ws);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    }
    delete ctx;
    return SOAPGB_OK;
}

const char *soapgb_last_error(const soapgb_ctx *ctx) {
    if (!ctx) return "null context";
    return ctx->err.c_str();
}

int soapgb_set_stream(soapgb_ctx *ctx, void *cuda_stream) {
    if (!ctx) return SOAPGB_ERR_ARG;
    cudaStream_t next = cuda_stream ? (cudaStream_t)cuda_stream : ctx->own_stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(next, &cap) != cudaSuccess) {
        cudaGetLastError();
        cap = cudaStreamCaptureStatusNone;
    }
    // a stream being captured into a graph cannot wait on work outside the capture: its
    // caller orders the graph's launch after the context's earlier work
    if (next != ctx->stream && ctx->stream && cap == cudaStreamCaptureStatusNone) {
        // every call's work ends on the context's stream and may still be queued there,
        // using the context's scratch: the new stream starts after it
        SOAP_DEVICE(ctx);
        if (!ctx->switch_event)
            SOAP_CUDA(ctx, cudaEventCreateWithFlags(&ctx->switch_event, cudaEventDisableTiming));
        SOAP_CUDA(ctx, cudaEventRecord(ctx->switch_event, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamWaitEvent(next, ctx->switch_event, 0));
    }
    ctx->stream = next;
    return SOAPGB_OK;
}

int soapgb_synchronize(soapgb_ctx *ctx) {
    if (!ctx) return SOAPGB_ERR_ARG;
    SOAP_DEVICE(ctx);
    SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return check_status(ctx, "soapgb_synchronize");
}

long long soapgb_launch_count(const soapgb_ctx *ctx) { return ctx ? ctx->launches : -1; }

int soapgb_set_compensated(soapgb_ctx *ctx, int on) {
    if (!ctx) return SOAPGB_ERR_ARG;
    ctx->fir_compensated = (on != 0);
    return SOAPGB_OK;
}

}  // extern "C"
