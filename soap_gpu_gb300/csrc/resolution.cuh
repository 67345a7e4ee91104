// Convolution / normalisation entry points shared with the pipeline.
#pragma once
#include "internal.cuh"

namespace soapgb {
// reference half width: rndup(window * Delta_lambda_cpu(sigma_v, wave0) / (wave1 - wave0))
int conv_halfwidth(double wave0, double wave1, double sigma_v, double window);
size_t resolution_scratch_bytes(int form, int n, int n_eff, int n_spec);
// All pointers device.  Spectrum s (rows of spec_stride) uses base_b when
// b_every > 0 and s % b_every == b_every - 1, else base_a (may be null: A = spec).
// d_spec holds float spectra when spec_f32 (FP32 form only), else double
int resolution_device(soapgb_ctx *ctx, int form, int n, int n_eff, int n_spec, const double *d_wave, double wave0,
                      double wave1, double wave_last, const void *d_spec, int spec_f32, long long spec_stride,
                      const double *base_a, const double *base_b, int b_every, double sigma_v, double window,
                      double step_mult, double step_exp, double sentinel, double *d_out, long long out_stride,
                      double *d_minmax, char *scratch);

// The FP32 form in two steps, for callers that run the spectra in chunks: prepare
// convolves the base spectra and sets up the per-spectrum state of all n_spec spectra in
// scratch; run convolves and normalises spectra [s0, s1) (s0 a multiple of b_every) of
// the FP32 rows spec32 into d_out rows [s0, s1).
struct Res32 {
    int n, n_eff, n_spec, wid, halo, nbx, b_every;
    double sentinel;
    const double *base_a, *base_b, *cb_a, *cb_b;
    const float *b32a, *b32b, *c32a, *c32b;
    const char *p32;
    float *conv32;
    unsigned *mm32;
    unsigned long long *mm;
    float *fac, *blk;
    unsigned long long *mmz;   // exact extrema of a zero spectrum, per base: [base][min, max]
    int *blist;                // the non-zero spectra of a chunk (its convolution's row list)
    char *next;   // first scratch byte after the state
};
int resolution32_prepare(soapgb_ctx *ctx, int n, int n_eff, int n_spec, const double *d_wave, double wave0,
                         double wave1, double wave_last, const double *base_a, const double *base_b, int b_every,
                         double sigma_v, double window, double step_mult, double step_exp, double sentinel,
                         char *scratch, Res32 &R);
// the normalised rows of a zero spectrum for the n_types spectrum types (tot, flux,
// bconv with b_every 3): out[n_types][n_eff], the same values resolution32_run writes
int resolution32_zero_rows(soapgb_ctx *ctx, const Res32 &R, int n_types, double *out);
// the normalised rows of the zero spectra (with zero_spec / zero_host): written by the
// normalisation (NORM), or not at all, the caller having them already (SKIP)
enum class ZeroRows { NORM, SKIP };
int resolution32_run(soapgb_ctx *ctx, const Res32 &R, const float *spec32, long long spec_stride, int s0, int s1,
                     double *d_out, long long out_stride, double *d_minmax,
                     const unsigned char *zero_spec = nullptr,    // [n_spec] device: 1 = spectrum known to be zero
                     const unsigned char *zero_host = nullptr,    // the same flags on the host (both or neither)
                     ZeroRows zero_rows = ZeroRows::NORM,
                     const int *blist_pre = nullptr,   // device list of the non-zero spectra of [s0, s1), by the caller
                     int nlist_pre = 0);
}  // namespace soapgb
