// Allocation-free convolution + normalisation entry point.
//
// soapgb_lower_resolution draws its scratch (the raw convolution of every spectrum
// and the per-spectrum min/max words) from the context's workspace, which it grows
// with cudaMalloc when a call needs more.  Some callers cannot allow that: an
// application whose device memory is owned by another allocator (a framework's
// caching pool or a fixed arena reserved at start-up) cannot have a library take
// memory behind its back, and a latency-critical loop cannot absorb a cudaMalloc /
// cudaFree pair, which synchronises the device.  This variant runs the same PLAIN64
// kernels with their scratch in a fixed array that lives in this file.
#include <mutex>

#include "internal.cuh"
#include "resolution.cuh"

using namespace soapgb;

// Scratch shared by every call on a device.  Every GPU that loads the library holds
// it until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[SOAPGB_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_scratch_ptr[kMaxDevices] = {nullptr};

// The array's device address, looked up once per device with that device current.
// In host code the array's name is only a host-side stand-in, so kernels are given
// this address instead.
int scratch_address(soapgb_ctx *ctx, unsigned char **out) {
    if (ctx->device < 0 || ctx->device >= kMaxDevices)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_lower_resolution_noalloc: device %d out of range", ctx->device);
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[ctx->device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_check(ctx, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_scratch_ptr[ctx->device] = (unsigned char *)p;
    }
    *out = g_scratch_ptr[ctx->device];
    return SOAPGB_OK;
}
}  // namespace

extern "C" size_t soapgb_noalloc_capacity(int n_eff) {
    // the largest spectrum count whose scratch, by the same byte count the call checks
    // (the PLAIN64 scratch does not depend on n), fits in the array; the count grows
    // with the spectra, so a bisection finds it
    if (n_eff <= 0) return 0;
    auto fits = [n_eff](size_t s) {
        return resolution_scratch_bytes(SOAPGB_PLAIN64, n_eff, n_eff, (int)s) <= (size_t)SOAPGB_NOALLOC_SCRATCH_BYTES;
    };
    if (!fits(1)) return 0;
    size_t lo = 1, hi = (size_t)SOAPGB_NOALLOC_SCRATCH_BYTES / sizeof(double) + 1;   // fits(lo), !fits(hi)
    while (hi - lo > 1) {
        size_t mid = lo + (hi - lo) / 2;
        (fits(mid) ? lo : hi) = mid;
    }
    return lo;
}

extern "C" int soapgb_lower_resolution_noalloc(soapgb_ctx *ctx, int n, int n_eff, int n_spec, const double *wave,
                                               const double *base, const double *spec, double sigma_v, double window,
                                               double step_mult, double step_exp, double sentinel, double *out,
                                               double *minmax_out) {
    if (!ctx) return SOAPGB_ERR_ARG;
    if (n < 3 || n_eff < 1 || n_eff > n || n_spec < 0 || !wave || !spec || !out || !(sigma_v > 0) ||
        !(step_exp > 0))
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_lower_resolution_noalloc: bad arguments");
    if (n_spec == 0) return SOAPGB_OK;
    size_t need = resolution_scratch_bytes(SOAPGB_PLAIN64, n, n_eff, n_spec);
    if (need > (size_t)SOAPGB_NOALLOC_SCRATCH_BYTES)
        return set_error(ctx, SOAPGB_ERR_ARG,
                         "soapgb_lower_resolution_noalloc: %d spectra of %d pixels need %zu scratch bytes, more than "
                         "the fixed %d (at most %zu spectra of this length per call)",
                         n_spec, n_eff, need, (int)SOAPGB_NOALLOC_SCRATCH_BYTES, soapgb_noalloc_capacity(n_eff));
    SOAP_DEVICE(ctx);
    unsigned char *scratch = nullptr;
    int rc = scratch_address(ctx, &scratch);
    if (rc) return rc;
    // the half width needs wave[0] and wave[1] on the host: they are read back (one
    // synchronisation) the first time this context sees the array and kept, and later
    // calls with the same array confirm them on the device instead (status 51 through
    // soapgb_synchronize when the array has changed)
    double w3[3];
    rc = wave_edges(ctx, SOAPGB_DEVICE, wave, n, n_eff, w3);
    if (rc) return rc;
    int wid = conv_halfwidth(w3[0], w3[1], sigma_v, window);
    if (wid < 1 || 2 * wid + 2 >= n)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_lower_resolution_noalloc: half width %d invalid for n=%d", wid, n);
    // the PLAIN64 kernels write every convolution value and initialise the min/max
    // words themselves, so nothing left in the array by an earlier call is read
    return resolution_device(ctx, SOAPGB_PLAIN64, n, n_eff, n_spec, wave, w3[0], w3[1], w3[2], spec, 0, n, base,
                             nullptr, 0, sigma_v, window, step_mult, step_exp, sentinel, out, n_eff, minmax_out,
                             (char *)scratch);
}
