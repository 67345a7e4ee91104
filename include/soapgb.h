/*
 * soapgb.h -- C ABI of libsoapgb, the GB300 (sm_103a) engine for SOAP-GPU's
 * per-phase spectral synthesis.
 *
 * Conventions
 *  - Every entry point returns an int status (SOAPGB_OK == 0).  On failure the
 *    context keeps a message, readable with soapgb_last_error().
 *  - Buffers are owned by the caller.  `mem` says where ALL the array arguments of
 *    one call live: SOAPGB_HOST (the library copies in and out through its own
 *    device workspace, inside the call) or SOAPGB_DEVICE (device pointers on the
 *    context's device; nothing is copied).  Host-mode calls return after the
 *    results are in host memory; device-mode calls are asynchronous on the
 *    context's stream (soapgb_synchronize() waits).
 *  - Arrays are row-major float64 unless stated; a "cube" is n_mu rows of n
 *    pixels, row b holding mu bin b.  n is the pixel count of the wavelength grid
 *    and n_eff = floor(n / 512) * 512 the number of pixels the reference processes
 *    and writes (it launches n/512 blocks of 512 threads).
 *  - One context = one device + one CUDA stream; a context must not be used from
 *    two host threads at once.  Each call makes the context's device current while
 *    it runs and gives the calling thread its previous current device back before it
 *    returns.
 *
 * Each function names the reference code it replaces (paths relative to the
 * reference's SOAP_code/ directory).  The reference exposes these steps as
 * separate executables driven through argv and float64 .bin files by
 * run_all_SOAP.py; the drop-in executables built from soap_gpu_gb300/csrc/tools
 * keep that argv/file contract on top of this ABI.
 */
#ifndef SOAPGB_H
#define SOAPGB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SOAPGB_OK 0
#define SOAPGB_ERR_ARG 1       /* invalid argument / size */
#define SOAPGB_ERR_CUDA 2      /* CUDA runtime error */
#define SOAPGB_ERR_ALLOC 3     /* device or host allocation failed */
#define SOAPGB_ERR_NUMERIC 4   /* fit failed / non-finite result */
#define SOAPGB_ERR_DEVICE 5    /* a kernel reported an error through its status word */

#define SOAPGB_HOST 0
#define SOAPGB_DEVICE 1

/* arithmetic forms of the integration kernels */
#define SOAPGB_PLAIN64 0  /* per-cell FP64, the reference's arithmetic and cell order */
#define SOAPGB_FAST64 1   /* collapsed shift-FIR in FP64 (same function, re-associated) */
#define SOAPGB_FAST32 2   /* collapsed shift-FIR in FP32 with compensated (Kahan) sums;
                             FP64 for Doppler factors, grid positions, tap weights */

typedef struct soapgb_ctx soapgb_ctx;

/* Star / disk parameters, as run_all_SOAP.py forwards them to SOAP_initialize
 * (run_all_SOAP.py:226-229, SOAP_initialize.cu:513-537). */
typedef struct {
    int grid;            /* disk grid side G */
    double period;       /* rotation period [d] */
    double omega_ratio;  /* differential rotation W_ratio */
    double incl;         /* inclination [deg] */
    double radius_km;    /* stellar radius [km] */
    double u1, u2;       /* quadratic limb darkening */
    double lb[4];        /* facula limb-brightening cubic LB0..LB3 */
} soapgb_star;

/* Per-cell disk maps (G*G each, iy-major: k = iy*G + iz).  Invisible cells hold
 * -999 (region 0), as written by SOAP_initialize.cu:399-422. */
typedef struct {
    double *delta;       /* rotational velocity [km/s] */
    double *limb;        /* limb darkening */
    double *mu;          /* mu = cos(theta) */
    int *region;         /* mu-bin index into the cubes */
    double *lb;          /* facula limb brightening */
} soapgb_maps;

/* Seed spectra (run_all_SOAP.py:94-100): n_mu x n each. */
typedef struct {
    const double *q_norm;    /* quiet, continuum-normalised  (new_noconti_convec_T_eff_T*) */
    const double *q_sed;     /* quiet, with continuum        (new_conti_convec_T_eff_T*)   */
    const double *spot_norm; /* spot, normalised             (new_noconti_convec_T_eff_Ts) */
    const double *fac_norm;  /* facula, normalised           (new_noconti_convec_T_eff_Tf) */
    const double *spot_sed;  /* spot continuum, row 0 used   (new_conti_T_eff_Ts)          */
    const double *fac_sed;   /* facula continuum, row 0 used (new_conti_T_eff_Tf)          */
    int n_mu;
} soapgb_cubes;

/* Temperatures forwarded to SOAP_integration (SOAP_integration.cu:469-497). */
typedef struct {
    int t_star;
    int t_diff_spot;
    int t_diff_fac;
    int nrho;            /* rim points per region (config [main] nrho) */
    int solar;           /* 1: facula intensity is a Planck ratio (SOAP_integration_solar.cu:433) */
} soapgb_activity;

/* ---- context ------------------------------------------------------------ */
int soapgb_ctx_create(int device, soapgb_ctx **out);
int soapgb_ctx_destroy(soapgb_ctx *ctx);
const char *soapgb_last_error(const soapgb_ctx *ctx);
/* Use an external CUDA stream (cudaStream_t passed as void*); NULL restores the
 * context's own stream, a non-blocking stream that is not ordered with the legacy
 * default stream.  A caller whose work is on the legacy default stream (torch's
 * default stream, handle 0) passes cudaStreamLegacy.  Switching streams orders the
 * new stream after the work the context queued on the previous one, except for a
 * stream that is being captured into a CUDA graph (it cannot wait on work outside the
 * capture): the caller then orders the graph's launches after that work. */
int soapgb_set_stream(soapgb_ctx *ctx, void *cuda_stream);
int soapgb_synchronize(soapgb_ctx *ctx);
/* Number of kernel launches issued by this context since creation. */
long long soapgb_launch_count(const soapgb_ctx *ctx);
/* Summation of the FP32 form's per-phase integration (no counterpart in the reference,
 * whose sums are FP64).  Every cell's terms are summed per work unit (cells of one mu
 * bin and class in a tile) in FP32 and each unit's deficit is rounded once; on = 1 (the
 * default) adds those unit deficits, about 9 per pixel and tile, in compensated (Kahan)
 * sums, on = 0 in plain FP32 sums. */
int soapgb_set_compensated(soapgb_ctx *ctx, int on);
/* Library version string. */
const char *soapgb_version(void);

/* Per-kernel tracing.  The reference times each process with std::chrono and prints
 * the wall time (SOAP_initialize.cu:603-604, SOAP_integration.cu:852-853,
 * SOAP_resolution.cu:433-434); here CUDA events bracket the library's kernel launches
 * on the context's stream while tracing is on.  soapgb_trace_enable(ctx, on) starts or
 * stops recording (and drops what was recorded); soapgb_trace_report synchronizes the
 * stream and writes one line per kernel, "name launches total_ms\n", in first-launch
 * order, then clears the record. */
int soapgb_trace_enable(soapgb_ctx *ctx, int on);
int soapgb_trace_report(soapgb_ctx *ctx, char *buf, size_t len);

/* ---- a3: disk maps ------------------------------------------------------
 * Replaces the grid part of itot, SOAP_initialize.cu:297-395 (and the map files
 * written at :399-422).  mu_boundary: n_mu-1 descending boundaries; a cell takes
 * the first bin k with mu > mu_boundary[k], else the last bin. */
int soapgb_disk_maps(soapgb_ctx *ctx, const soapgb_star *star, int n_mu,
                     const double *mu_boundary, int mem, soapgb_maps *maps_out);

/* ---- a4-a7: quiet-star disk integration ---------------------------------
 * Replaces itot's cell loop, SOAP_initialize.cu:339-395 (fast_shift,
 * fast_interp_new, fast_sum at :117-176): sum over visible cells (iy-major order)
 * of the cell's Doppler-shifted, linearly interpolated, limb-darkened cube row.
 * sum_out: n values ([n_eff, n) set to 0).  `step` is the grid step passed as
 * argv[10] of SOAP_initialize. */
int soapgb_quiet_disk(soapgb_ctx *ctx, int form, int n, int n_eff, const double *wave,
                      const double *cube, int n_mu, int grid, const double *delta,
                      const double *limb, const int *region, double step, int mem,
                      double *sum_out);

/* ---- a8 / a14: instrumental convolution + normalisation -----------------
 * Replaces lower_resolution_gpu, SOAP_initialize.cu:446-505 (quiet) and
 * SOAP_resolution.cu:235-310 (per phase and type).  For each of n_spec spectra
 * A_s = base - spec_s (base may be NULL: A_s = spec_s), all n long with zero tail:
 *   C_s[i] = sum_{m=i-w}^{i+w-2} step_mult (1 - A_s[m]) e^{-(m-i)^2 step_exp^2 / (2 s_i^2)} / (s_i sqrt(2 pi))
 *   for w < i < n-1-w and i < n_eff, with w = rndup(window * dl_f32(sigma_v, wave[0]) / (wave[1]-wave[0]))
 *   out_s[i] = 1 - C_s[i] (1 - min A_s) / max(sentinel, max_{C != 0} C_s),  i < n_eff.
 * The reference hard-codes step_mult = step_exp = 0.005 in SOAP_resolution and
 * step_exp = 0.005 in SOAP_initialize; sentinel is its -60000 start value.
 * out: n_spec x n_eff.  minmax_out (optional, host or device like the rest):
 * n_spec x 2 (min A, max C). */
int soapgb_lower_resolution(soapgb_ctx *ctx, int form, int n, int n_eff, int n_spec,
                            const double *wave, const double *base, const double *spec,
                            double sigma_v, double window, double step_mult, double step_exp,
                            double sentinel, int mem, double *out, double *minmax_out);

/* Adjoint of soapgb_lower_resolution in the PLAIN64 arithmetic (the differentiable
 * form; the reference has no counterpart).  Same arguments as the forward plus g_out
 * (n_spec x n_eff), the gradient of a scalar w.r.t. out.  Writes grad_spec
 * (n_spec x n), its gradient w.r.t. spec, and -- when grad_base is not NULL, which
 * needs a base -- grad_base (n), w.r.t. base summed over the spectra.  The
 * normalisation's min A and max C are differentiated at the first pixel holding each
 * (a maximum that stayed at the sentinel carries no gradient).  Deterministic: every
 * sum runs in a fixed order, without atomics. */
int soapgb_lower_resolution_adjoint(soapgb_ctx *ctx, int n, int n_eff, int n_spec,
                                    const double *wave, const double *base, const double *spec,
                                    double sigma_v, double window, double step_mult, double step_exp,
                                    double sentinel, const double *g_out, int mem,
                                    double *grad_spec, double *grad_base);

/* ---- a9-a10: per-phase temperature and type maps -------------------------
 * Replaces spot_init_gpu / spot_phase_gpu / spot_area / spot_scan and the region
 * loop, SOAP_integration.cu:21-161,326-390,686-785.  regions: rows of
 * (lat, long, size, type) -- type 0 spot, 1 facula -- phase p uses rows
 * [reg_offsets[p], reg_offsets[p+1]) applied in order (later rows overwrite).
 * temp/bi: n_phase x G*G, -9999 where no region. */
int soapgb_phase_maps(soapgb_ctx *ctx, int grid, double incl, int n_phase,
                      const double *phases, const int *reg_offsets, const double *regions,
                      const soapgb_activity *act, int mem, double *temp, double *bi);

/* ---- a11-a12: per-phase active-region integration ------------------------
 * Replaces spot_integrate, SOAP_integration.cu:392-447 (+ fast_flux / fast_bconv /
 * fast_tot / fast_intensity(_fac) at :285-323): for every active cell of every
 * phase, in iy-major order,
 *   flux += s - I q,  bconv += q - a,  tot += s - I a
 * with q, s, a the shifted rows of q_norm, q_sed and spot_norm|fac_norm.
 * flux/bconv/tot: n_phase x n each ([n_eff, n) set to 0). */
int soapgb_phase_integrate(soapgb_ctx *ctx, int form, int n, int n_eff, const double *wave,
                           int grid, int n_phase, const double *temp, const double *bi,
                           const soapgb_maps *maps, const soapgb_cubes *cubes, double step,
                           const soapgb_activity *act, int mem,
                           double *flux, double *bconv, double *tot);

/* Adjoint of soapgb_phase_integrate in the PLAIN64 arithmetic (the differentiable
 * form; the reference has no counterpart).  Given the gradients g_flux, g_bconv, g_tot
 * (n_phase x n each) of a scalar with respect to the three outputs, writes its
 * gradients with respect to the four cubes (n_mu x n each), the two continuum rows
 * (spot_sed, fac_sed: n each), the limb map and the velocity map (G*G each), each
 * summed over the phases.  The outputs are linear in the cubes, rows and limb values;
 * in a cell's velocity they are continuous and piecewise smooth (the derivative of the
 * interpolation weight inside each owner interval).  Chain rules: dL/du1 = -(1 - mu),
 * dL/du2 = -(1 - mu)^2 on visible cells; the velocity map is proportional to vsini.
 * g_flux and g_tot may both be NULL, meaning zero (a scalar of bconv alone): the
 * continuum-row gradients are then zero and cost no pass.
 * Deterministic: every sum runs in a fixed order, without atomics. */
int soapgb_phase_integrate_adjoint(soapgb_ctx *ctx, int n, int n_eff, const double *wave,
                                   int grid, int n_phase, const double *temp, const double *bi,
                                   const soapgb_maps *maps, const soapgb_cubes *cubes, double step,
                                   const soapgb_activity *act, const double *g_flux,
                                   const double *g_bconv, const double *g_tot, int mem,
                                   double *grad_q_norm, double *grad_q_sed, double *grad_spot_norm,
                                   double *grad_fac_norm, double *grad_spot_sed, double *grad_fac_sed,
                                   double *grad_limb, double *grad_delta);

/* ---- a15-a16: mask CCF ---------------------------------------------------
 * Replaces calculate_CCF_1 / calc_mask / calculate_CCF_2, CCF_func.py:5-91, with
 * the extended grid of run_all_SOAP.py:292-295.  wave_trim: the n_w trimmed
 * wavelengths; lines filtered by the caller (run_all_SOAP.py:288).  mask_step and
 * index_old are the literals 0.005 and 20000 of CCF_func.py:8-9,62-63 (pass the
 * real step and int(wave_extend/step) for other grids).  spectra: n_spec x n_w;
 * ccf_out: n_spec x n_v raw sums.  If `normalise` is set each CCF is divided by its
 * max and apodised as run_all_SOAP.py:306-314.  form: PLAIN64 / FAST64 sum in FP64;
 * FAST32 multiplies in FP32 and sums with compensation (FP64 assembly). */
int soapgb_ccf(soapgb_ctx *ctx, int form, int n_v, const double *vel, int n_lines,
               const double *line_wave, const double *line_weight, int n_w,
               const double *wave_trim, double step_size, double wave_extend,
               double mask_step, int index_old, int n_spec, const double *spectra,
               int normalise, int mem, double *ccf_out);

/* Adjoint of soapgb_ccf in FP64 (the differentiable form; the reference has no
 * counterpart).  Same mask arguments as the forward; g_ccf (n_spec x n_v) is the
 * gradient of a scalar w.r.t. ccf_out.  With `normalise` set, ccf_raw (n_spec x n_v)
 * holds the forward's raw sums (soapgb_ccf with normalise = 0) and the max is
 * differentiated at its first index.  Writes grad_spectra (n_spec x n_w).  Deterministic:
 * one thread per pixel sums the velocities in order, without atomics. */
int soapgb_ccf_adjoint(soapgb_ctx *ctx, int n_v, const double *vel, int n_lines,
                       const double *line_wave, const double *line_weight, int n_w,
                       const double *wave_trim, double step_size, double wave_extend,
                       double mask_step, int index_old, int n_spec, const double *ccf_raw,
                       int normalise, const double *g_ccf, int mem, double *grad_spectra);

/* ---- a17-a18: Gaussian fit + bisector -------------------------------------
 * Replaces BIS_FIT2.cpp:97-317 (GSL trust-region Levenberg-Marquardt fit of
 * c + k exp(-(x-x0)^2 / 2 sigma^2), then the 91-depth bisector and its span), for
 * n_spec CCFs at once.  x: n velocities [m/s] shared by all; y, err: n_spec x n
 * (err may be NULL for unit errors).  Outputs per spectrum: model[n],
 * par[5] = (c, |k|, span, v0, fwhm), depth[91], bis[91]; iters (optional int per
 * spectrum, < 0 when the fit did not converge). */
int soapgb_gauss_bis(soapgb_ctx *ctx, int n_spec, int n, const double *x, const double *y,
                     const double *err, int mem, double *model, double *par, double *depth,
                     double *bis, int *iters);

/* Adjoint of the Gaussian fit of soapgb_gauss_bis (the differentiable form; the
 * reference has no counterpart), by the implicit function theorem at the fitted
 * optimum: H dtheta/dy = J^T W with H the full Hessian of the residual sum of squares
 * (Gauss-Newton term plus the residual-weighted second derivatives).  x, y, err as
 * for the fit; model and par are its outputs; g_par (n_spec x 5) holds the gradient
 * of a scalar w.r.t. par = (c, |k|, span, v0, fwhm).  The bisector span
 * (BIS_FIT2.cpp:214-268) is differentiated with its per-depth crossing intervals held
 * fixed (a discrete choice, like the region coverage): through the normalised CCF
 * directly and through the fit's parameters.  Writes grad_y (n_spec x n).  A singular
 * system gives a zero gradient for that spectrum and the status SOAPGB_ERR_DEVICE. */
int soapgb_gauss_fit_adjoint(soapgb_ctx *ctx, int n_spec, int n, const double *x, const double *y,
                             const double *err, const double *model, const double *par,
                             const double *g_par, int mem, double *grad_y);

/* ---- composite: the per-phase stages in one call --------------------------
 * Runs a9-a14 for every phase: maps, integration, convolution and normalisation of
 * the three deficit spectra against the quiet spectra.  quiet_sed / quiet_norm are
 * the n-long disk sums of a4-a7 (tail zero).  lower: n_phase x 3 x n_eff, types in
 * the order tot, flux, bconv (SOAP_resolution.cu:414-416); raw (optional):
 * n_phase x 3 x n_eff deficit spectra in the same order.  conv_step is the step
 * used in the Gaussian (0.005 in the reference binaries).
 * With mem = SOAPGB_DEVICE the descriptors phases, reg_offsets and regions may be
 * host or device memory: from host memory the call does not synchronise, so calls
 * queue on the stream back to back.  wave[0], wave[1] and wave[n_eff - 1] of a device
 * wavelength array are read (one synchronisation) the first time the array is seen
 * and kept in the context; later calls confirm them on the device, and a changed
 * array is reported by soapgb_synchronize (status 51). */
int soapgb_phase_pipeline(soapgb_ctx *ctx, int form, int n, int n_eff, const double *wave,
                          const soapgb_star *star, const soapgb_maps *maps,
                          const soapgb_cubes *cubes, double step, const soapgb_activity *act,
                          int n_phase, const double *phases, const int *reg_offsets,
                          const double *regions, const double *quiet_sed,
                          const double *quiet_norm, double sigma_v, double conv_step,
                          double sentinel, int mem, double *lower, double *raw);

/* ---- batched form: many stars in one job ---------------------------------
 * Replaces one run_all_SOAP.py invocation per star (run_all_SOAP.py:226-250: two
 * SOAP_initialize runs, then SOAP_integration's phase loop, SOAP_integration.cu:661-845,
 * and SOAP_resolution) for a batch of stars of uneven grids, regions and phase counts
 * that share the seed spectra and the wavelength grid.  FP32 form only.  Per star the
 * run builds the disk maps (a3), the two quiet spectra (a4-a7), the region maps' lists
 * (a9-a10) and tile plans; the active-region integration (a11-a12) of every visible
 * phase of every star is ONE persistent launch over (star, phase, tile) items; then each
 * star's three deficit spectra per phase are convolved and normalised against its own
 * quiet spectra (a14).
 * soapgb_batch_create does the host-side work once (region tables, visibility, sizes),
 * allocates the batch's device memory (soapgb_batch_device_bytes) and uploads the
 * descriptors; it synchronises the context's stream.  soapgb_batch_run only enqueues
 * device work on the context's stream (and streams it joins back), reads no host memory,
 * allocates nothing and does not synchronise, so a caller may capture it in a CUDA graph;
 * lower (device) receives total phases x 3 x n_eff spectra (tot, flux, bconv), star s's
 * phases at rows [phase_offsets[s], phase_offsets[s + 1]); quiet (optional, device)
 * n_star x 2 x n (quiet with continuum, normalised quiet).  The device arrays named in the
 * descriptor (wave, the cubes) must stay valid while the batch is used.
 * chunk and blocks_per_sm shape the integration launch's walk: its (star, phase, tile)
 * positions are dealt to the blocks round robin in chunks of `chunk` positions (0: one
 * contiguous share per block), with at most blocks_per_sm blocks per SM (0: as many as
 * fit); soapgb_batch_tune changes them for later runs. */
typedef struct soapgb_batch soapgb_batch;
typedef struct {
    int form;                    /* SOAPGB_FAST32 */
    int n, n_eff;                /* the shared wavelength grid */
    const double *wave;          /* n, device */
    const soapgb_cubes *cubes;   /* the shared seed cubes, device */
    const double *mu_boundary;   /* n_mu - 1, host */
    double step;                 /* grid step */
    soapgb_activity act;         /* temperatures, rim points, solar variant (shared) */
    double sigma_v, conv_step, sentinel;
    int n_star;
    const soapgb_star *stars;    /* n_star, host */
    const int *phase_offsets;    /* n_star + 1, host */
    const double *phases;        /* phase_offsets[n_star], host */
    const int *reg_offsets;      /* phase_offsets[n_star] + 1, host: region rows of each phase */
    const double *regions;       /* rows (lat, long, size, type), host */
    int chunk;
    int blocks_per_sm;
} soapgb_batch_desc;
int soapgb_batch_create(soapgb_ctx *ctx, const soapgb_batch_desc *desc, soapgb_batch **out);
int soapgb_batch_run(soapgb_ctx *ctx, soapgb_batch *batch, double *lower, double *quiet);
int soapgb_batch_tune(soapgb_batch *batch, int chunk, int blocks_per_sm);
size_t soapgb_batch_device_bytes(const soapgb_batch *batch);
/* number of (star, phase) items with a visible region, the integration launch's phases */
long long soapgb_batch_items(const soapgb_batch *batch);
int soapgb_batch_destroy(soapgb_batch *batch);

/* ---- bisector injection of the seed spectra --------------------------------
 * Replaces BIS_inject_spectral_quiet / BIS_inject_spectral_active
 * (CB_injection_faculae.py:191-244, with Delta_wavelength :119-123), which the
 * reference runs in a Python loop over pixels once per seed spectrum and mu bin.
 * For every mu bin b < n_mu, pixel k of flux moves by the relativistic shift of
 * rv_b(flux[k]) and the spectrum is re-sampled on wave: linear interpolation as
 * scipy's interp1d does it (numpy.interp), 0 outside the shifted range.  out is
 * n_mu x n.  Polynomials have n_coef (<= 16) coefficients per bin, highest power
 * first (numpy.poly1d), rows of n_mu x n_coef.
 *   SOAPGB_BIS_QUIET:  rv = poly(coeffs_b)(f) * scale.
 *   SOAPGB_BIS_ACTIVE: rv = (poly(coeffs_b)(f) + vshift_b) * scale for 0.5 < f < dep_cut_b,
 *     (poly(coeffs_low_b)(f) + vshift_b) * scale for f <= 0.5,
 *     (vcut_b + vshift_b) * scale for f > dep_cut_b, and no shift otherwise.
 * A shifted grid that does not increase is an error (device status 61), where the
 * reference's interp1d would sort it. */
#define SOAPGB_BIS_QUIET 0
#define SOAPGB_BIS_ACTIVE 1
int soapgb_bisector_inject(soapgb_ctx *ctx, int mode, int n, int n_mu, int n_coef, const double *wave,
                           const double *flux, const double *coeffs, const double *coeffs_low,
                           const double *dep_cut, const double *vcut, const double *vshift, double scale,
                           int mem, double *out);

/* ---- allocation-free convolution + normalisation --------------------------
 * No counterpart in the reference: an extra entry point of this library.  The
 * same computation as soapgb_lower_resolution in the PLAIN64 form, for callers
 * that must not have the library allocate device memory -- an application whose
 * device memory belongs to another allocator (a framework's caching pool or an
 * arena reserved at start-up), or a latency-bound loop that cannot absorb the
 * device-wide synchronisation of cudaMalloc / cudaFree.  Its scratch is a fixed
 * SOAPGB_NOALLOC_SCRATCH_BYTES array in the library's device image, held by every
 * GPU that loads the library until the process exits; soapgb_noalloc_capacity(n_eff)
 * gives how many spectra of n_eff pixels fit in one call (a call with exactly that
 * many is accepted), and larger requests are rejected with SOAPGB_ERR_ARG.  All
 * array arguments are device pointers.  The first call on a device looks up the
 * array's device address (a cudaGetSymbolAddress call with that device current), and
 * the first call of a context with a given wavelength array reads wave[0], wave[1]
 * and wave[n_eff - 1] back to the host, which synchronises the context's stream;
 * later calls with the same array do not synchronise (a one-thread kernel confirms
 * the kept values, and soapgb_synchronize reports status 51 if the array changed).
 * Make those first calls before any stream capture.  Calls share the array: two
 * calls whose work overlaps on the GPU (different streams or contexts on one
 * device) race on it. */
#define SOAPGB_NOALLOC_SCRATCH_BYTES (8 * 1024 * 1024)
size_t soapgb_noalloc_capacity(int n_eff);
int soapgb_lower_resolution_noalloc(soapgb_ctx *ctx, int n, int n_eff, int n_spec, const double *wave,
                                    const double *base, const double *spec, double sigma_v,
                                    double window, double step_mult, double step_exp,
                                    double sentinel, double *out, double *minmax_out);

#ifdef __cplusplus
}
#endif
#endif /* SOAPGB_H */
