// soapgb_torch: libsoapgb's calls for the differentiable and batched forms as torch operators.
//
// torch.ops.soapgb.* take the context handle (the soapgb_ctx pointer as an int, from
// soap_gpu_gb300.api.Context), CUDA tensors (float64 / int32, contiguous) and scalars,
// allocate their outputs with torch on the inputs' device, and run on torch's current
// stream.  They are the device-buffer calls of include/soapgb.h, one operator per entry
// point; an error status raises with the library's message.
#include <torch/extension.h>
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>

#include <cstdint>
#include <optional>
#include <tuple>
#include <vector>

#include "soapgb.h"

namespace {

using at::Tensor;

soapgb_ctx *as_ctx(int64_t h) {
    TORCH_CHECK(h != 0, "soapgb: null context");
    return reinterpret_cast<soapgb_ctx *>(static_cast<uintptr_t>(h));
}

void check(soapgb_ctx *ctx, int rc, const char *what) {
    TORCH_CHECK(rc == SOAPGB_OK, "soapgb error ", rc, " in ", what, ": ", soapgb_last_error(ctx));
}

// the context on torch's current stream of `ref`'s device (the legacy default stream,
// handle 0, is passed as cudaStreamLegacy: 0 means the context's own stream)
soapgb_ctx *on_stream(int64_t h, const Tensor &ref) {
    soapgb_ctx *ctx = as_ctx(h);
    TORCH_CHECK(ref.is_cuda(), "soapgb: CUDA tensors expected");
    cudaStream_t s = c10::cuda::getCurrentCUDAStream(ref.device().index()).stream();
    check(ctx, soapgb_set_stream(ctx, s ? (void *)s : (void *)cudaStreamLegacy), "soapgb_set_stream");
    return ctx;
}

const double *f64(const Tensor &t, const char *name) {
    TORCH_CHECK(t.is_cuda() && t.scalar_type() == at::kDouble && t.is_contiguous(), "soapgb: ", name,
                " must be a contiguous CUDA float64 tensor");
    return t.data_ptr<double>();
}
const double *f64_opt(const std::optional<Tensor> &t, const char *name) {
    return (t.has_value() && t->defined()) ? f64(*t, name) : nullptr;
}
const int *i32(const Tensor &t, const char *name) {
    TORCH_CHECK(t.is_cuda() && t.scalar_type() == at::kInt && t.is_contiguous(), "soapgb: ", name,
                " must be a contiguous CUDA int32 tensor");
    return t.data_ptr<int>();
}
Tensor empty64(const Tensor &like, at::IntArrayRef shape) {
    return at::empty(shape, like.options().dtype(at::kDouble));
}

soapgb_activity activity(const std::vector<int64_t> &a) {
    TORCH_CHECK(a.size() == 5, "soapgb: activity is (t_star, t_diff_spot, t_diff_fac, nrho, solar)");
    soapgb_activity act;
    act.t_star = (int)a[0];
    act.t_diff_spot = (int)a[1];
    act.t_diff_fac = (int)a[2];
    act.nrho = (int)a[3];
    act.solar = (int)a[4];
    return act;
}

soapgb_maps maps_of(const Tensor &delta, const Tensor &limb, const Tensor &region, const Tensor &lb) {
    soapgb_maps m;
    m.delta = const_cast<double *>(f64(delta, "delta"));
    m.limb = const_cast<double *>(f64(limb, "limb"));
    m.mu = nullptr;
    m.region = const_cast<int *>(i32(region, "region"));
    m.lb = const_cast<double *>(f64(lb, "lb"));
    return m;
}

soapgb_cubes cubes_of(const Tensor &q_norm, const Tensor &q_sed, const Tensor &spot_norm, const Tensor &fac_norm,
                      const Tensor &spot_sed, const Tensor &fac_sed) {
    TORCH_CHECK(q_norm.dim() == 2, "soapgb: the cubes are n_mu x n");
    soapgb_cubes c;
    c.q_norm = f64(q_norm, "q_norm");
    c.q_sed = f64(q_sed, "q_sed");
    c.spot_norm = f64(spot_norm, "spot_norm");
    c.fac_norm = f64(fac_norm, "fac_norm");
    c.spot_sed = f64(spot_sed, "spot_sed");
    c.fac_sed = f64(fac_sed, "fac_sed");
    c.n_mu = (int)q_norm.size(0);
    return c;
}

// ---- a3: disk maps (delta, limb, mu, lb, region), each G*G --------------------
std::tuple<Tensor, Tensor, Tensor, Tensor, Tensor> disk_maps(int64_t h, int64_t grid, double period,
                                                             double omega_ratio, double incl, double radius_km,
                                                             double u1, double u2, const Tensor &mu_boundary,
                                                             std::vector<double> lb) {
    c10::cuda::CUDAGuard guard(mu_boundary.device());
    soapgb_ctx *ctx = on_stream(h, mu_boundary);
    TORCH_CHECK(lb.size() == 4, "soapgb: lb is the cubic LB0..LB3");
    soapgb_star st;
    st.grid = (int)grid;
    st.period = period;
    st.omega_ratio = omega_ratio;
    st.incl = incl;
    st.radius_km = radius_km;
    st.u1 = u1;
    st.u2 = u2;
    for (int q = 0; q < 4; ++q) st.lb[q] = lb[q];
    const int64_t gm = grid * grid;
    Tensor delta = empty64(mu_boundary, {gm}), limb = empty64(mu_boundary, {gm}), mu = empty64(mu_boundary, {gm}),
           lbm = empty64(mu_boundary, {gm});
    Tensor region = at::empty({gm}, mu_boundary.options().dtype(at::kInt));
    soapgb_maps m{delta.data_ptr<double>(), limb.data_ptr<double>(), mu.data_ptr<double>(), region.data_ptr<int>(),
                  lbm.data_ptr<double>()};
    const int n_mu = (int)mu_boundary.numel() + 1;
    check(ctx, soapgb_disk_maps(ctx, &st, n_mu, mu_boundary.numel() ? f64(mu_boundary, "mu_boundary") : nullptr,
                                SOAPGB_DEVICE, &m),
          "soapgb_disk_maps");
    return {delta, limb, mu, lbm, region};
}

// ---- a4-a7: quiet-star disk integration -------------------------------------------
Tensor quiet_disk(int64_t h, int64_t form, const Tensor &wave, const Tensor &cube, int64_t n_eff, int64_t grid,
                  const Tensor &delta, const Tensor &limb, const Tensor &region, double step) {
    c10::cuda::CUDAGuard guard(wave.device());
    soapgb_ctx *ctx = on_stream(h, wave);
    const int n = (int)wave.numel();
    const int n_mu = cube.dim() == 2 ? (int)cube.size(0) : 1;
    Tensor out = empty64(wave, {n});
    check(ctx, soapgb_quiet_disk(ctx, (int)form, n, (int)n_eff, f64(wave, "wave"), f64(cube, "cube"), n_mu, (int)grid,
                                 f64(delta, "delta"), f64(limb, "limb"), i32(region, "region"), step, SOAPGB_DEVICE,
                                 out.data_ptr<double>()),
          "soapgb_quiet_disk");
    return out;
}

// ---- a11-a12: per-phase integration and its adjoint --------------------------------
std::tuple<Tensor, Tensor, Tensor> phase_integrate(int64_t h, int64_t form, const Tensor &wave, int64_t n_eff,
                                                   int64_t grid, const Tensor &temp, const Tensor &bi,
                                                   const Tensor &delta, const Tensor &limb, const Tensor &region,
                                                   const Tensor &lbm, const Tensor &q_norm, const Tensor &q_sed,
                                                   const Tensor &spot_norm, const Tensor &fac_norm,
                                                   const Tensor &spot_sed, const Tensor &fac_sed, double step,
                                                   std::vector<int64_t> act_v) {
    c10::cuda::CUDAGuard guard(wave.device());
    soapgb_ctx *ctx = on_stream(h, wave);
    const int n = (int)wave.numel();
    const int n_phase = (int)temp.size(0);
    soapgb_maps m = maps_of(delta, limb, region, lbm);
    soapgb_cubes c = cubes_of(q_norm, q_sed, spot_norm, fac_norm, spot_sed, fac_sed);
    soapgb_activity act = activity(act_v);
    Tensor flux = empty64(wave, {n_phase, n}), bconv = empty64(wave, {n_phase, n}), tot = empty64(wave, {n_phase, n});
    check(ctx, soapgb_phase_integrate(ctx, (int)form, n, (int)n_eff, f64(wave, "wave"), (int)grid, n_phase,
                                      f64(temp, "temp"), f64(bi, "bi"), &m, &c, step, &act, SOAPGB_DEVICE,
                                      flux.data_ptr<double>(), bconv.data_ptr<double>(), tot.data_ptr<double>()),
          "soapgb_phase_integrate");
    return {flux, bconv, tot};
}

// gradients (q_norm, q_sed, spot_norm, fac_norm, spot_sed, fac_sed, limb, delta); g_flux and
// g_tot may both be None (bconv alone: the continuum rows' pass is skipped)
std::vector<Tensor> phase_integrate_adjoint(int64_t h, const Tensor &wave, int64_t n_eff, int64_t grid,
                                            const Tensor &temp, const Tensor &bi, const Tensor &delta,
                                            const Tensor &limb, const Tensor &region, const Tensor &lbm,
                                            const Tensor &q_norm, const Tensor &q_sed, const Tensor &spot_norm,
                                            const Tensor &fac_norm, const Tensor &spot_sed, const Tensor &fac_sed,
                                            double step, std::vector<int64_t> act_v,
                                            const std::optional<Tensor> &g_flux, const Tensor &g_bconv,
                                            const std::optional<Tensor> &g_tot) {
    c10::cuda::CUDAGuard guard(wave.device());
    soapgb_ctx *ctx = on_stream(h, wave);
    const int n = (int)wave.numel();
    const int n_phase = (int)temp.size(0);
    const int64_t gm = grid * grid;
    soapgb_maps m = maps_of(delta, limb, region, lbm);
    soapgb_cubes c = cubes_of(q_norm, q_sed, spot_norm, fac_norm, spot_sed, fac_sed);
    soapgb_activity act = activity(act_v);
    const int64_t n_mu = c.n_mu;
    std::vector<Tensor> g = {empty64(wave, {n_mu, n}), empty64(wave, {n_mu, n}), empty64(wave, {n_mu, n}),
                             empty64(wave, {n_mu, n}), empty64(wave, {n}),       empty64(wave, {n}),
                             empty64(wave, {gm}),      empty64(wave, {gm})};
    check(ctx, soapgb_phase_integrate_adjoint(
                   ctx, n, (int)n_eff, f64(wave, "wave"), (int)grid, n_phase, f64(temp, "temp"), f64(bi, "bi"), &m, &c,
                   step, &act, f64_opt(g_flux, "g_flux"), f64(g_bconv, "g_bconv"), f64_opt(g_tot, "g_tot"),
                   SOAPGB_DEVICE, g[0].data_ptr<double>(), g[1].data_ptr<double>(), g[2].data_ptr<double>(),
                   g[3].data_ptr<double>(), g[4].data_ptr<double>(), g[5].data_ptr<double>(),
                   g[6].data_ptr<double>(), g[7].data_ptr<double>()),
          "soapgb_phase_integrate_adjoint");
    return g;
}

// ---- a8 / a14: convolution + normalisation and its adjoint --------------------------
std::tuple<Tensor, Tensor> lower_resolution(int64_t h, int64_t form, const Tensor &wave, const Tensor &spec,
                                            int64_t n_eff, double sigma_v, const std::optional<Tensor> &base,
                                            double window, double step_mult, double step_exp, double sentinel) {
    c10::cuda::CUDAGuard guard(wave.device());
    soapgb_ctx *ctx = on_stream(h, wave);
    TORCH_CHECK(spec.dim() == 2, "soapgb: spec is n_spec x n");
    const int n = (int)wave.numel(), n_spec = (int)spec.size(0);
    Tensor out = empty64(wave, {n_spec, n_eff}), mm = empty64(wave, {n_spec, 2});
    check(ctx, soapgb_lower_resolution(ctx, (int)form, n, (int)n_eff, n_spec, f64(wave, "wave"), f64_opt(base, "base"),
                                       f64(spec, "spec"), sigma_v, window, step_mult, step_exp, sentinel,
                                       SOAPGB_DEVICE, out.data_ptr<double>(), mm.data_ptr<double>()),
          "soapgb_lower_resolution");
    return {out, mm};
}

std::tuple<Tensor, std::optional<Tensor>> lower_resolution_adjoint(int64_t h, const Tensor &wave, const Tensor &spec,
                                                                   int64_t n_eff, double sigma_v, const Tensor &g_out,
                                                                   const std::optional<Tensor> &base, double window,
                                                                   double step_mult, double step_exp,
                                                                   double sentinel, bool want_base) {
    c10::cuda::CUDAGuard guard(wave.device());
    soapgb_ctx *ctx = on_stream(h, wave);
    const int n = (int)wave.numel(), n_spec = (int)spec.size(0);
    Tensor gs = empty64(wave, {n_spec, n});
    std::optional<Tensor> gb;
    const bool with_base = want_base && base.has_value() && base->defined();
    if (with_base) gb = empty64(wave, {n});
    check(ctx, soapgb_lower_resolution_adjoint(ctx, n, (int)n_eff, n_spec, f64(wave, "wave"), f64_opt(base, "base"),
                                               f64(spec, "spec"), sigma_v, window, step_mult, step_exp, sentinel,
                                               f64(g_out, "g_out"), SOAPGB_DEVICE, gs.data_ptr<double>(),
                                               with_base ? gb->data_ptr<double>() : nullptr),
          "soapgb_lower_resolution_adjoint");
    return {gs, gb};
}

// ---- a15-a16: mask CCF and its adjoint ----------------------------------------------
Tensor ccf(int64_t h, int64_t form, const Tensor &vel, const Tensor &line_wave, const Tensor &line_weight,
           const Tensor &wave_trim, double step_size, const Tensor &spectra, bool normalise, double wave_extend,
           double mask_step, int64_t index_old) {
    c10::cuda::CUDAGuard guard(spectra.device());
    soapgb_ctx *ctx = on_stream(h, spectra);
    TORCH_CHECK(spectra.dim() == 2, "soapgb: spectra is n_spec x n_w");
    const int n_spec = (int)spectra.size(0), n_v = (int)vel.numel();
    Tensor out = empty64(spectra, {n_spec, n_v});
    check(ctx, soapgb_ccf(ctx, (int)form, n_v, f64(vel, "vel"), (int)line_wave.numel(), f64(line_wave, "line_wave"),
                          f64(line_weight, "line_weight"), (int)wave_trim.numel(), f64(wave_trim, "wave_trim"),
                          step_size, wave_extend, mask_step, (int)index_old, n_spec, f64(spectra, "spectra"),
                          normalise ? 1 : 0, SOAPGB_DEVICE, out.data_ptr<double>()),
          "soapgb_ccf");
    return out;
}

Tensor ccf_adjoint(int64_t h, const Tensor &vel, const Tensor &line_wave, const Tensor &line_weight,
                   const Tensor &wave_trim, double step_size, const Tensor &g_ccf,
                   const std::optional<Tensor> &ccf_raw, bool normalise, double wave_extend, double mask_step,
                   int64_t index_old) {
    c10::cuda::CUDAGuard guard(g_ccf.device());
    soapgb_ctx *ctx = on_stream(h, g_ccf);
    const int n_spec = (int)g_ccf.size(0), n_v = (int)vel.numel(), n_w = (int)wave_trim.numel();
    Tensor out = empty64(g_ccf, {n_spec, n_w});
    check(ctx, soapgb_ccf_adjoint(ctx, n_v, f64(vel, "vel"), (int)line_wave.numel(), f64(line_wave, "line_wave"),
                                  f64(line_weight, "line_weight"), n_w, f64(wave_trim, "wave_trim"), step_size,
                                  wave_extend, mask_step, (int)index_old, n_spec, f64_opt(ccf_raw, "ccf_raw"),
                                  normalise ? 1 : 0, f64(g_ccf, "g_ccf"), SOAPGB_DEVICE, out.data_ptr<double>()),
          "soapgb_ccf_adjoint");
    return out;
}

// ---- a17-a18: Gaussian fit + bisector and the fit's adjoint ------------------------------
// (model n_spec x n, par n_spec x 5, depth and bis n_spec x 91, iterations n_spec)
std::tuple<Tensor, Tensor, Tensor, Tensor, Tensor> gauss_bis(int64_t h, const Tensor &x, const Tensor &y,
                                                             const std::optional<Tensor> &err) {
    c10::cuda::CUDAGuard guard(y.device());
    soapgb_ctx *ctx = on_stream(h, y);
    TORCH_CHECK(y.dim() == 2, "soapgb: y is n_spec x n");
    const int n_spec = (int)y.size(0), n = (int)x.numel();
    Tensor model = empty64(y, {n_spec, n}), par = empty64(y, {n_spec, 5}), depth = empty64(y, {n_spec, 91}),
           bis = empty64(y, {n_spec, 91});
    Tensor iters = at::empty({n_spec}, y.options().dtype(at::kInt));
    check(ctx, soapgb_gauss_bis(ctx, n_spec, n, f64(x, "x"), f64(y, "y"), f64_opt(err, "err"), SOAPGB_DEVICE,
                                model.data_ptr<double>(), par.data_ptr<double>(), depth.data_ptr<double>(),
                                bis.data_ptr<double>(), iters.data_ptr<int>()),
          "soapgb_gauss_bis");
    return {model, par, depth, bis, iters};
}

Tensor gauss_fit_adjoint(int64_t h, const Tensor &x, const Tensor &y, const Tensor &model, const Tensor &par,
                         const Tensor &g_par, const std::optional<Tensor> &err) {
    c10::cuda::CUDAGuard guard(y.device());
    soapgb_ctx *ctx = on_stream(h, y);
    const int n_spec = (int)y.size(0), n = (int)x.numel();
    Tensor out = empty64(y, {n_spec, n});
    check(ctx, soapgb_gauss_fit_adjoint(ctx, n_spec, n, f64(x, "x"), f64(y, "y"), f64_opt(err, "err"),
                                        f64(model, "model"), f64(par, "par"), f64(g_par, "g_par"), SOAPGB_DEVICE,
                                        out.data_ptr<double>()),
          "soapgb_gauss_fit_adjoint");
    return out;
}

// ---- batched form: one run of a batch made by soapgb_batch_create -----------------------
// out: (total phases, 3, n_eff), allocated here when None; quiet: the stars' quiet
// spectra (optional output, as soapgb_batch_run takes it)
Tensor batch_run(int64_t h, int64_t batch, int64_t total_phases, int64_t n_eff, int64_t device,
                 const std::optional<Tensor> &out, const std::optional<Tensor> &quiet) {
    TORCH_CHECK(batch != 0, "soapgb: null batch");
    Tensor o = (out.has_value() && out->defined())
                   ? *out
                   : at::empty({total_phases, 3, n_eff},
                               at::TensorOptions().dtype(at::kDouble).device(at::kCUDA, (c10::DeviceIndex)device));
    TORCH_CHECK(o.numel() == total_phases * 3 * n_eff, "soapgb: out is (total phases, 3, n_eff)");
    c10::cuda::CUDAGuard guard(o.device());
    soapgb_ctx *ctx = on_stream(h, o);
    check(ctx, soapgb_batch_run(ctx, reinterpret_cast<soapgb_batch *>(static_cast<uintptr_t>(batch)),
                                const_cast<double *>(f64(o, "out")),
                                const_cast<double *>(f64_opt(quiet, "quiet"))),
          "soapgb_batch_run");
    return o;
}

// waits for the context's stream and raises a device status (a singular fit system)
void synchronize(int64_t h) {
    soapgb_ctx *ctx = as_ctx(h);
    check(ctx, soapgb_synchronize(ctx), "soapgb_synchronize");
}

}  // namespace

TORCH_LIBRARY(soapgb, m) {
    m.def("disk_maps(int ctx, int grid, float period, float omega_ratio, float incl, float radius_km, float u1, "
          "float u2, Tensor mu_boundary, float[] lb) -> (Tensor, Tensor, Tensor, Tensor, Tensor)",
          disk_maps);
    m.def("quiet_disk(int ctx, int form, Tensor wave, Tensor cube, int n_eff, int grid, Tensor delta, Tensor limb, "
          "Tensor region, float step) -> Tensor",
          quiet_disk);
    m.def("phase_integrate(int ctx, int form, Tensor wave, int n_eff, int grid, Tensor temp, Tensor bi, "
          "Tensor delta, Tensor limb, Tensor region, Tensor lb, Tensor q_norm, Tensor q_sed, Tensor spot_norm, "
          "Tensor fac_norm, Tensor spot_sed, Tensor fac_sed, float step, int[] act) -> (Tensor, Tensor, Tensor)",
          phase_integrate);
    m.def("phase_integrate_adjoint(int ctx, Tensor wave, int n_eff, int grid, Tensor temp, Tensor bi, "
          "Tensor delta, Tensor limb, Tensor region, Tensor lb, Tensor q_norm, Tensor q_sed, Tensor spot_norm, "
          "Tensor fac_norm, Tensor spot_sed, Tensor fac_sed, float step, int[] act, Tensor? g_flux, "
          "Tensor g_bconv, Tensor? g_tot) -> Tensor[]",
          phase_integrate_adjoint);
    m.def("lower_resolution(int ctx, int form, Tensor wave, Tensor spec, int n_eff, float sigma_v, Tensor? base, "
          "float window, float step_mult, float step_exp, float sentinel) -> (Tensor, Tensor)",
          lower_resolution);
    m.def("lower_resolution_adjoint(int ctx, Tensor wave, Tensor spec, int n_eff, float sigma_v, Tensor g_out, "
          "Tensor? base, float window, float step_mult, float step_exp, float sentinel, bool want_base) "
          "-> (Tensor, Tensor?)",
          lower_resolution_adjoint);
    m.def("ccf(int ctx, int form, Tensor vel, Tensor line_wave, Tensor line_weight, Tensor wave_trim, "
          "float step_size, Tensor spectra, bool normalise, float wave_extend, float mask_step, int index_old) "
          "-> Tensor",
          ccf);
    m.def("ccf_adjoint(int ctx, Tensor vel, Tensor line_wave, Tensor line_weight, Tensor wave_trim, "
          "float step_size, Tensor g_ccf, Tensor? ccf_raw, bool normalise, float wave_extend, float mask_step, "
          "int index_old) -> Tensor",
          ccf_adjoint);
    m.def("gauss_bis(int ctx, Tensor x, Tensor y, Tensor? err) -> (Tensor, Tensor, Tensor, Tensor, Tensor)",
          gauss_bis);
    m.def("gauss_fit_adjoint(int ctx, Tensor x, Tensor y, Tensor model, Tensor par, Tensor g_par, Tensor? err) "
          "-> Tensor",
          gauss_fit_adjoint);
    m.def("batch_run(int ctx, int batch, int total_phases, int n_eff, int device, Tensor? out, Tensor? quiet) "
          "-> Tensor",
          batch_run);
    m.def("synchronize(int ctx) -> ()", synchronize);
}
