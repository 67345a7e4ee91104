// Velocity order of the disk cells for the collapsed shift-FIR (fir.cu).
//
// The collapsed form groups cells by their integer shift at every tile; with the
// visible cells sorted by (mu bin, v == 0, Doppler slope) the cells sharing a shift
// form contiguous ranges at every tile, so a tile finds its groups by binary search
// instead of visiting every cell.  The order comes from two stable radix sorts (CUB,
// the CUDA toolkit's template library): by slope, then by (mu bin, v == 0).
#include <algorithm>

#include <cub/device/device_radix_sort.cuh>

#include "fir.cuh"

namespace soapgb {

size_t fir_sort_temp_bytes(long long gm) {
    size_t b64 = 0, b32 = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, b64, (const unsigned long long *)nullptr, (unsigned long long *)nullptr,
                                    (const int *)nullptr, (int *)nullptr, (int)gm);
    cub::DeviceRadixSort::SortPairs(nullptr, b32, (const unsigned *)nullptr, (unsigned *)nullptr,
                                    (const int *)nullptr, (int *)nullptr, (int)gm);
    return std::max(b64, b32);
}

// library kernels: not counted in the context's launch counter
int fir_sort_u64(soapgb_ctx *ctx, long long gm, const unsigned long long *keys_in, unsigned long long *keys_out,
                 const int *vals_in, int *vals_out, void *temp, size_t temp_bytes) {
    size_t bytes = temp_bytes;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(temp, bytes, keys_in, keys_out, vals_in, vals_out, (int)gm, 0, 64,
                                                    ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, "cell sort (slope)");
    return SOAPGB_OK;
}

int fir_sort_u32(soapgb_ctx *ctx, long long gm, const unsigned *keys_in, unsigned *keys_out, const int *vals_in,
                 int *vals_out, int end_bit, void *temp, size_t temp_bytes) {
    size_t bytes = temp_bytes;
    cudaError_t e = cub::DeviceRadixSort::SortPairs(temp, bytes, keys_in, keys_out, vals_in, vals_out, (int)gm, 0,
                                                    end_bit, ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, "cell sort (mu bin)");
    return SOAPGB_OK;
}

}  // namespace soapgb
