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
}  // namespace soapgb
