/*
 * ORACLE -- test infrastructure only.
 *
 * Plain-C restatement of the reference SOAP-GPU per-phase synthesis path.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this
 * file's shared library, and only as the checker: the product path is the CUDA
 * library under soap_gpu_gb300/ and never calls into here.
 *
 * Every function cites the reference file:line it follows (paths relative to the
 * reference project root, SOAP_code/).  Two semantics are provided where the
 * reference's GPU code is nondeterministic or reads memory it never wrote:
 *
 *   SEM_GATHER  ("patched"): every output pixel j takes the unique shifted source
 *               interval [x_i, x_{i+1}) that contains it (owner i in [0, n_eff-2]);
 *               pixels without an owner are 0; every fresh buffer is zero.  This is
 *               the deterministic semantics the CUDA library implements.
 *   SEM_SCATTER ("as written"): the reference's own scatter, one write per source
 *               at ceil(x_i), holes keep the previous cell's value, collisions are
 *               resolved "higher source index wins", buffers start at zero and the
 *               uninitialised shift slot lambda'[n_eff] reads 0.  Used only to
 *               compare with outputs of the unmodified reference binaries.
 *
 * Build: gcc -O2 -fPIC -shared -fopenmp -ffp-contract=off (no FMA contraction, so
 * x86 and Arm hosts give identical bits).  Parity is pinned against the reference's
 * own CCF_func.py / run_all_SOAP.py functions (tests/golden) and against outputs of
 * the reference CUDA binaries run on the GPU host.  The Gaussian fit restates GSL's
 * trust-region Levenberg-Marquardt (GSL is not vendored): that part is pinned only
 * against scipy's MINPACK optimum, i.e. "parity unpinned" with respect to GSL.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define C_LIGHT 299792458.
#define PI_REF 3.141592653589793238463

enum { SEM_GATHER = 0, SEM_SCATTER = 1 };

/* ------------------------------------------------------------------------- */
/* small helpers                                                               */
/* ------------------------------------------------------------------------- */

/* SOAP_initialize.cu:19-36 rndup(n, nb_decimal) */
static double orc_rndup(double n, int nb_decimal)
{
    double t = n * pow(10, nb_decimal) - floor(n * pow(10, nb_decimal));
    if (t >= 0.5) {
        n *= pow(10, nb_decimal);
        n = ceil(n);
        n /= pow(10, nb_decimal);
    } else {
        n *= pow(10, nb_decimal);
        n = floor(n);
        n /= pow(10, nb_decimal);
    }
    return n;
}

/* SOAP_initialize.cu:39-50 Delta_lambda_cpu: note the float sqrtf */
double orc_delta_lambda_cpu(double line_width, double lambda_line0)
{
    double beta = line_width / C_LIGHT;
    return -1 * lambda_line0 * (1 - (double)sqrtf((float)((1 + beta) / (1 - beta))));
}

/* SOAP_initialize.cu:55-66 Delta_lambda (device, double sqrt) */
static double orc_delta_lambda(double line_width, double lambda_line0)
{
    double beta = line_width / C_LIGHT;
    return -1 * lambda_line0 * (1 - sqrt((1 + beta) / (1 - beta)));
}

/* convolution half width: SOAP_initialize.cu:449-450, SOAP_resolution.cu:243-244 */
int orc_conv_halfwidth(const double *wave, double sigma_v, double window_width)
{
    double wavelength_step = wave[1] - wave[0];
    return (int)orc_rndup((window_width * orc_delta_lambda_cpu(sigma_v, wave[0])) / wavelength_step, 0);
}

/* ------------------------------------------------------------------------- */
/* a3: disk maps  (SOAP_initialize.cu:297-395, grid part of itot)             */
/* ------------------------------------------------------------------------- */
void orc_disk_maps(int grid, double period, double omega_ratio, double incl_deg,
                   double radius_star, double limba1, double limba2,
                   int n_mu, const double *mu_boundary,
                   double lb0, double lb1, double lb2, double lb3,
                   double *delta_maps, double *limb_maps, double *mu_maps,
                   int *region_maps, double *lb_maps)
{
    double incl = incl_deg * PI_REF / 180.;
    double delta_grid = 2. / grid;
    double theta_grid = 180.0 / grid;
    double omega0 = 360.0 / period;
    double omega1 = omega0 * omega_ratio;
    for (int iy = 0; iy < grid; iy++) {
        double y = -1. + iy * delta_grid;
        for (int iz = 0; iz < grid; iz++) {
            double z = -1. + iz * delta_grid;
            double theta_z = -90.0 + iz * theta_grid;
            double s = sin(theta_z * PI_REF / 180);
            double omega_velo = (omega0 + omega1 * (s * s)) * PI_REF / (180 * 24 * 3600) * radius_star;
            double delta = y * omega_velo * sin(incl);
            int k = iy * grid + iz;
            delta_maps[k] = -999.0;
            limb_maps[k] = -999.0;
            mu_maps[k] = -999.0;
            lb_maps[k] = -999.0;
            region_maps[k] = 0;
            if ((y * y + z * z) <= 1.) {
                /* pow(x, .5) in the reference; sqrt is the correctly rounded form */
                double r_cos = sqrt(1. - (y * y + z * z));
                double limb = 1. - limba1 * (1 - r_cos) - limba2 * (1 - r_cos) * (1 - r_cos);
                double lb = lb0 + lb1 * r_cos + lb2 * r_cos * r_cos + lb3 * r_cos * r_cos * r_cos;
                /* SOAP_initialize.cu:370-377: first boundary below mu; the reference
                 * reads one entry past the boundary array for the last bin, the
                 * patched default is the last bin. */
                int spec_idx = n_mu - 1;
                for (int id_mu = 0; id_mu < n_mu - 1; id_mu++) {
                    if (r_cos > mu_boundary[id_mu]) { spec_idx = id_mu; break; }
                }
                delta_maps[k] = delta;
                limb_maps[k] = limb;
                mu_maps[k] = r_cos;
                region_maps[k] = spec_idx;
                lb_maps[k] = lb;
            }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* a4/a6: one cell's shifted, interpolated, limb-darkened spectrum            */
/* SOAP_initialize.cu:117-167 (fast_shift, fast_interp_new)                   */
/* ------------------------------------------------------------------------- */

/* shifted source position x_i (in grid index units) and its ceil, exactly as
 * fast_interp_new computes new_index (SOAP_initialize.cu:145) */
static inline long orc_ceil_pos(long i, double fbeta, double lambda0, double step)
{
    double x = (double)i * (1 + fbeta) + fbeta * lambda0 / step;
    return (long)ceil(x);
}

/* out[0..n_eff) for one cell.  For SEM_GATHER out is overwritten entirely; for
 * SEM_SCATTER only the written pixels change (out keeps its previous content). */
static void orc_cell_interp(int sem, int n, int n_eff, const double *lambda,
                            const double *row, double delta, double limb,
                            double step, double *lshift, double *out)
{
    double lambda0 = lambda[0];
    double beta = delta * 1000. / C_LIGHT;
    double fbeta = -1 * (1 - sqrt((1 + beta) / (1 - beta)));
    if (sem == SEM_GATHER) {
        if (delta == 0.0) {               /* SOAP_initialize.cu:149-152 */
            for (int j = 0; j < n_eff; j++) out[j] = row[j] * limb;
            return;
        }
        #pragma omp parallel for schedule(static)
        for (int i = 0; i < n_eff; i++)   /* fast_shift, SOAP_initialize.cu:125 */
            lshift[i] = lambda[i] + orc_delta_lambda(delta * 1000., lambda[i]);
        #pragma omp parallel for schedule(static)
        for (int j = 0; j < n_eff; j++) out[j] = 0.0;
        /* every source i owns the pixels [ceil(x_i), ceil(x_{i+1})): disjoint ranges,
         * so the sources can be processed in parallel */
        #pragma omp parallel for schedule(static)
        for (int i = 0; i < n_eff - 1; i++) {
            long c_lo = orc_ceil_pos(i, fbeta, lambda0, step);
            long c_hi = orc_ceil_pos(i + 1, fbeta, lambda0, step);
            long j0 = c_lo < 0 ? 0 : c_lo;
            long j1 = c_hi > n_eff ? n_eff : c_hi;
            if (j0 < j1) {
                double g = row[i + 1] - row[i];     /* spec_grad_2d */
                double d = lshift[i + 1] - lshift[i];
                for (long j = j0; j < j1; j++)
                    out[j] = (row[i] + g / d * (lambda[j] - lshift[i])) * limb;
            }
        }
        return;
    }
    /* SEM_SCATTER: the reference as written (lshift has n+1 slots) */
    if (delta == 0.0) {
        for (int j = 0; j < n_eff; j++) out[j] = row[j] * limb;
        return;
    }
    for (int i = 0; i < n_eff; i++)
        lshift[i] = lambda[i] + orc_delta_lambda(delta * 1000., lambda[i]);
    lshift[n_eff] = 0.0;                    /* never written by fast_shift */
    for (int i = 0; i < n_eff; i++) {
        long j = orc_ceil_pos(i, fbeta, lambda0, step);
        if (j < 0 || j >= n) continue;      /* v<0 guard; v>0 writes past n dropped */
        double g = (i + 1 < n) ? row[i + 1] - row[i] : 0.0;
        out[j] = (row[i] + g / (lshift[i + 1] - lshift[i]) * (lambda[j] - lshift[i])) * limb;
    }
}

/* ------------------------------------------------------------------------- */
/* a4-a7: quiet-star disk integration (SOAP_initialize.cu:297-395)            */
/* cube: n_mu x n row-major, sum_out: n (tail [n_eff, n) stays 0)             */
/* ------------------------------------------------------------------------- */
void orc_quiet_disk(int sem, int n, int n_eff, const double *lambda, const double *cube,
                    int grid, const double *delta_maps, const double *limb_maps,
                    const int *region_maps, double step, double *sum_out)
{
    double *lshift = (double *)calloc((size_t)n + 1, sizeof(double));
    double *tmp = (double *)calloc((size_t)n, sizeof(double));
    for (int j = 0; j < n; j++) sum_out[j] = 0.0;
    for (int k = 0; k < grid * grid; k++) {
        if (limb_maps[k] == -999.0) continue;   /* invisible cell */
        const double *row = cube + (size_t)region_maps[k] * n;
        orc_cell_interp(sem, n, n_eff, lambda, row, delta_maps[k], limb_maps[k], step, lshift, tmp);
        #pragma omp parallel for schedule(static)
        for (int j = 0; j < n_eff; j++) sum_out[j] = sum_out[j] + tmp[j];   /* fast_sum */
    }
    free(lshift);
    free(tmp);
}

/* ------------------------------------------------------------------------- */
/* a8/a14: Gaussian instrument convolution, min/max, normalisation            */
/* SOAP_initialize.cu:69-96,206-294,437-505; SOAP_resolution.cu:66-95,123-310 */
/*   a[n]      : the spectrum A (tail [n_eff, n) must be 0)                   */
/*   conv_out  : optional n_eff raw convolution C                               */
/*   out[n_eff]: 1 - C (1 - min A) / max_{C != 0} C                            */
/* ------------------------------------------------------------------------- */
void orc_lower_resolution(int n, int n_eff, const double *wave, const double *a,
                          double sigma_v, double window_width, double step_mult,
                          double step_exp, double sentinel, double *conv_out,
                          double *out, double *minmax_out)
{
    int wid = orc_conv_halfwidth(wave, sigma_v, window_width);
    double pi = PI_REF;
    double *c = (double *)calloc((size_t)n, sizeof(double));
    #pragma omp parallel for schedule(static)
    for (int index = 0; index < n_eff; index++) {
        double sig = orc_delta_lambda(sigma_v, wave[index]);     /* wav_sigma */
        double acc = 0.0;
        if ((index > wid) && (index + wid < n - 1)) {
            for (int m = index - wid; m < index + wid - 1; m++) {
                int d = m - index;
                acc += step_mult * (1.0 - a[m]) * 1. / (sig * sqrt(2. * pi)) *
                       exp(-d * d * step_exp * step_exp / (2 * sig * sig));
            }
        }
        c[index] = acc;
    }
    double maxv = sentinel;                   /* reduceMaxIdxOptimizedShared */
    for (int i = 0; i < n; i++)
        if (c[i] != 0.0 && maxv < c[i]) maxv = c[i];
    double minv = a[0];                       /* reduceMinIdxOptimizedShared */
    for (int i = 0; i < n; i++)
        if (minv > a[i]) minv = a[i];
    for (int i = 0; i < n_eff; i++) {         /* spec_norm */
        out[i] = 1.0 - c[i] * (1 - minv) / maxv;
        if (conv_out) conv_out[i] = c[i];
    }
    if (minmax_out) { minmax_out[0] = minv; minmax_out[1] = maxv; }
    free(c);
}

/* ------------------------------------------------------------------------- */
/* a9: region rim, phase rotation and bounding box                             */
/* SOAP_integration.cu:125-161 spot_init_gpu, :21-47 spot_phase_gpu,          */
/* :51-120 spot_area (computed sequentially: one consistent view of all rim    */
/* points instead of the reference's cross-block race)                         */
/* bounds: [iminy, iminz, imaxy, imaxz, visible]                               */
/* ------------------------------------------------------------------------- */
void orc_region_bbox(double s, double longitude, double latitude, double inclination,
                     int nrho, double phase, int grid, int *bounds)
{
    double lon = longitude * PI_REF / 180.;
    double lat = latitude * PI_REF / 180.;
    double inc = inclination * PI_REF / 180.;
    double rho_step = 2. * PI_REF / (nrho - 1);
    double b = -lat, g = lon, b2 = PI_REF / 2. - inc;
    double R[3][3] = {{cos(b2) * cos(g) * cos(b) - sin(b) * sin(b2), -sin(g) * cos(b2), cos(b2) * cos(g) * sin(b) + sin(b2) * cos(b)},
                      {sin(g) * cos(b), cos(g), sin(g) * sin(b)},
                      {-sin(b2) * cos(g) * cos(b) - cos(b2) * sin(b), sin(b2) * sin(g), -sin(b2) * cos(g) * sin(b) + cos(b2) * cos(b)}};
    double psi = -phase * (2 * PI_REF);
    double axe[3] = {cos(inc), 0, sin(inc)};
    double cp = cos(psi), sp = sin(psi);
    double P[3][3] = {{(1 - cp) * axe[0] * axe[0] + cp, (1 - cp) * axe[0] * axe[1] + sp * axe[2], (1 - cp) * axe[0] * axe[2] - sp * axe[1]},
                      {(1 - cp) * axe[1] * axe[0] - sp * axe[2], (1 - cp) * axe[1] * axe[1] + cp, (1 - cp) * axe[1] * axe[2] + sp * axe[0]},
                      {(1 - cp) * axe[2] * axe[0] + sp * axe[1], (1 - cp) * axe[2] * axe[1] - sp * axe[0], (1 - cp) * axe[2] * axe[2] + cp}};
    double grid_step = 2. / grid;
    double miny = 1, minz = 1, maxy = -1, maxz = -1;
    int sum_on = 0, sum_off = 0;
    for (int k = 0; k < nrho; k++) {
        double rho = -PI_REF + k * rho_step;
        double x2[3] = {sqrt(1 - s * s), s * cos(rho), s * sin(rho)};
        double x1[3], x3[3];
        for (int r = 0; r < 3; r++) x1[r] = R[r][0] * x2[0] + R[r][1] * x2[1] + R[r][2] * x2[2];
        for (int r = 0; r < 3; r++) x3[r] = P[r][0] * x1[0] + P[r][1] * x1[1] + P[r][2] * x1[2];
        if (x3[0] >= 0) {
            sum_on++;
            if (x3[1] < miny) miny = x3[1];
            if (x3[2] < minz) minz = x3[2];
            if (x3[1] > maxy) maxy = x3[1];
            if (x3[2] > maxz) maxz = x3[2];
        } else {
            sum_off++;
        }
    }
    if ((sum_on > 0) && (sum_off > 0)) {
        if (miny * maxy < 0) { if (minz < 0) minz = -1; else maxz = 1; }
        if (minz * maxz < 0) { if (miny < 0) miny = -1; else maxy = 1; }
    }
    bounds[0] = (int)floor((1. + miny) / grid_step);
    bounds[1] = (int)floor((1. + minz) / grid_step);
    bounds[2] = (int)ceil((1. + maxy) / grid_step);
    bounds[3] = (int)ceil((1. + maxz) / grid_step);
    bounds[4] = sum_on == 0 ? 0 : 1;
}

/* SOAP_integration.cu:164-202 spot_inverse_rotation, matrix part.  The reference
 * writes `--phase*(2*pi)`: phase is decremented by one before the multiply. */
void orc_inverse_rotation_matrix(double longitude, double latitude, double inclination,
                                 double phase, double *R3out)
{
    double g2 = (phase - 1.0) * (2 * PI_REF);
    double i = inclination * PI_REF / 180.;
    double b = latitude * PI_REF / 180.;
    double g = -longitude * PI_REF / 180.;
    double b2 = -(PI_REF / 2. - i);
    double R[3][3] = {{(1 - cos(g2)) * cos(i) * cos(i) + cos(g2), sin(g2) * sin(i), (1 - cos(g2)) * cos(i) * sin(i)},
                      {-sin(g2) * sin(i), cos(g2), sin(g2) * cos(i)},
                      {(1 - cos(g2)) * sin(i) * cos(i), -sin(g2) * cos(i), (1 - cos(g2)) * sin(i) * sin(i) + cos(g2)}};
    double R2[3][3] = {{cos(b) * cos(g) * cos(b2) - sin(b2) * sin(b), -sin(g) * cos(b), cos(b) * cos(g) * sin(b2) + sin(b) * cos(b2)},
                       {sin(g) * cos(b2), cos(g), sin(g) * sin(b2)},
                       {-sin(b) * cos(g) * cos(b2) - cos(b) * sin(b2), sin(b) * sin(g), -sin(b) * cos(g) * sin(b2) + cos(b) * cos(b2)}};
    for (int r = 0; r < 3; r++)
        for (int q = 0; q < 3; q++)
            R3out[r * 3 + q] = R2[r][0] * R[0][q] + R2[r][1] * R[1][q] + R2[r][2] * R[2][q];
}

/* ------------------------------------------------------------------------- */
/* a10: per-phase temperature / type maps (SOAP_integration.cu:326-390,       */
/* 686-785).  regions: n_reg rows of (lat, long, size, type), applied in order */
/* (later regions overwrite).  Bounding boxes are clamped to [0, grid].         */
/* ------------------------------------------------------------------------- */
void orc_phase_maps(int grid, int nrho, double incl, double phase, int n_reg,
                    const double *regions, int t_star, int t_diff_spot, int t_diff_fac,
                    double *temp_maps, double *bi_maps)
{
    int gm = grid * grid;
    for (int k = 0; k < gm; k++) { temp_maps[k] = -9999.0; bi_maps[k] = -9999.0; }
    double delta_grid = 2. / grid;
    for (int r = 0; r < n_reg; r++) {
        double lat = regions[4 * r + 0], lon = regions[4 * r + 1];
        double s = regions[4 * r + 2], type = regions[4 * r + 3];
        int bd[5];
        orc_region_bbox(s, lon, lat, incl, nrho, phase, grid, bd);
        if (bd[4] != 1) continue;
        double R3[9];
        orc_inverse_rotation_matrix(lon, lat, incl, phase, R3);
        int iy0 = bd[0] < 0 ? 0 : bd[0], iz0 = bd[1] < 0 ? 0 : bd[1];
        int iy1 = bd[2] > grid ? grid : bd[2], iz1 = bd[3] > grid ? grid : bd[3];
        for (int iy = iy0; iy < iy1; iy++) {
            double y = -1. + iy * delta_grid;
            for (int iz = iz0; iz < iz1; iz++) {
                double z = -1. + iz * delta_grid;
                if (z * z + y * y < 1.) {
                    double xa0 = sqrt(1. - (y * y + z * z));
                    double xi0 = R3[0] * xa0 + R3[1] * y + R3[2] * z;
                    if (xi0 * xi0 >= 1. - s * s) {
                        int k = iy * grid + iz;
                        double r_cos = xa0;
                        if (type == 0.0) {
                            int t_spot = t_star - t_diff_spot;
                            temp_maps[k] = t_spot;
                            bi_maps[k] = 0.0;
                        } else {
                            int t_plage = (int)(t_star + t_diff_fac + 0.9 - 407.7 * r_cos + 190.9 * (r_cos * r_cos));
                            temp_maps[k] = t_plage;
                            bi_maps[k] = 1.0;
                        }
                    }
                }
            }
        }
    }
}

/* SOAP_integration.cu:205-212 loi_Planck */
static double orc_planck(double lambda0, double temp)
{
    double c = 299792458.;
    double h = 6.62606896e-34;
    double k_b = 1.380e-23;
    double scale = 1e-10;
    return 2 * h * pow(c, 2) * 1. / pow(lambda0 * scale, 5) * 1. / (exp((h * c) / (lambda0 * k_b * temp * scale)) - 1);
}

/* ------------------------------------------------------------------------- */
/* a11-a12: per-phase active-region integration (SOAP_integration.cu:392-447) */
/* cubes: quiet normalised, quiet SED, spot normalised, facula normalised      */
/* (n_mu x n each); spot_sed / fac_sed: row 0 of the spot / facula continuum   */
/* cubes; outputs flux/bconv/tot: n each (tail stays 0)                        */
/* ------------------------------------------------------------------------- */
void orc_phase_integrate(int sem, int n, int n_eff, const double *lambda, int grid,
                         const double *temp_maps, const double *bi_maps,
                         const double *delta_maps, const double *limb_maps,
                         const int *region_maps, const double *lb_maps,
                         const double *q_norm, const double *q_sed,
                         const double *spot_norm, const double *fac_norm,
                         const double *spot_sed, const double *fac_sed,
                         double step, int solar, int t_star, int t_diff_fac,
                         double *flux, double *bconv, double *tot)
{
    double *lshift = (double *)calloc((size_t)n + 1, sizeof(double));
    double *q = (double *)calloc((size_t)n, sizeof(double));
    double *sv = (double *)calloc((size_t)n, sizeof(double));
    double *a = (double *)calloc((size_t)n, sizeof(double));
    double *inten = (double *)calloc((size_t)n, sizeof(double));
    for (int j = 0; j < n; j++) { flux[j] = 0.0; bconv[j] = 0.0; tot[j] = 0.0; }
    for (int k = 0; k < grid * grid; k++) {
        double bi = bi_maps[k];
        if (bi != 0.0 && bi != 1.0) continue;
        size_t off = (size_t)region_maps[k] * n;
        double d = delta_maps[k], l = limb_maps[k];
        orc_cell_interp(sem, n, n_eff, lambda, q_norm + off, d, l, step, lshift, q);
        orc_cell_interp(sem, n, n_eff, lambda, q_sed + off, d, l, step, lshift, sv);
        if (bi == 0.0) {
            int t_norm = (int)temp_maps[k];
            #pragma omp parallel for schedule(static)
            for (int j = 0; j < n_eff; j++)       /* fast_intensity */
                inten[j] = orc_planck(lambda[j], temp_maps[k]) / orc_planck(lambda[j], t_norm) * spot_sed[j];
            orc_cell_interp(sem, n, n_eff, lambda, spot_norm + off, d, l, step, lshift, a);
        } else {
            if (solar) {                          /* SOAP_integration_solar.cu:427,433 */
                int t_norm = (int)(t_star + t_diff_fac + 0.9 - 216.8);
                #pragma omp parallel for schedule(static)
                for (int j = 0; j < n_eff; j++)
                    inten[j] = orc_planck(lambda[j], temp_maps[k]) / orc_planck(lambda[j], t_norm) * fac_sed[j];
            } else {                              /* fast_intensity_fac */
                for (int j = 0; j < n_eff; j++) inten[j] = (1 + lb_maps[k]) * fac_sed[j];
            }
            orc_cell_interp(sem, n, n_eff, lambda, fac_norm + off, d, l, step, lshift, a);
        }
        #pragma omp parallel for schedule(static)
        for (int j = 0; j < n_eff; j++) {         /* fast_flux / fast_bconv / fast_tot */
            flux[j] = flux[j] + sv[j] - inten[j] * q[j];
            bconv[j] = bconv[j] + q[j] - a[j];
            tot[j] = tot[j] + sv[j] - a[j] * inten[j];
        }
    }
    free(lshift); free(q); free(sv); free(a); free(inten);
}

/* ------------------------------------------------------------------------- */
/* a15: CCF mask template (CCF_func.py:5-24 calculate_CCF_1, :39-91 calc_mask, */
/* wavelength_extend built as run_all_SOAP.py:292-295 with numpy.linspace).    */
/* M: n_v x n_w.  mask_step is the literal 0.005 of CCF_func.py:62-63;          */
/* index_old the literal 20000 of CCF_func.py:8-9.  Returns 0, or -1 when a     */
/* line's hole touches the extended array's ends or the slice size mismatches.  */
/* ------------------------------------------------------------------------- */
static double orc_linspace_at(double start, double stop, int num, int k)
{
    if (k == num - 1) return stop;
    double step = (stop - start) / (num - 1);
    return (double)k * step + start;
}

int orc_ccf_mask(int n_v, const double *vel, int n_lines, const double *line_wave,
                 const double *line_weight, int n_w, const double *wave_trim,
                 double step_size, double wave_extend, double mask_step, int index_old,
                 double *M)
{
    int np_ext = (int)(wave_extend / step_size);
    int n_ext = n_w + 2 * np_ext;
    if (n_ext - 2 * index_old != n_w) return -1;
    double wmin = wave_trim[0];
    for (int j = 1; j < n_w; j++) if (wave_trim[j] < wmin) wmin = wave_trim[j];
    double *we = (double *)malloc(sizeof(double) * (size_t)n_ext);
    double b_start = wmin - step_size * np_ext;
    double a_start = wave_trim[n_w - 1], a_stop = wave_trim[n_w - 1] + step_size * np_ext;
    for (int k = 0; k < np_ext; k++) we[k] = orc_linspace_at(b_start, wmin, np_ext, k);
    for (int k = 0; k < n_w; k++) we[np_ext + k] = wave_trim[k];
    for (int k = 0; k < np_ext; k++) we[np_ext + n_w + k] = orc_linspace_at(a_start, a_stop, np_ext, k);
    double begin_wave = we[0];
    for (int k = 1; k < n_ext; k++) if (we[k] < begin_wave) begin_wave = we[k];
    double *mask = (double *)malloc(sizeof(double) * (size_t)n_ext);
    double beta = 820. / C_LIGHT;
    int rc = 0;
    for (int iv = 0; iv < n_v && rc == 0; iv++) {
        for (int k = 0; k < n_ext; k++) mask[k] = 0.0;
        double fac = 1 + vel[iv] / C_LIGHT;
        for (int l = 0; l < n_lines; l++) {
            double ls = line_wave[l] * fac;
            double hw = ls * (sqrt((1 + beta) / (1 - beta)) - 1);
            double beg = ls - hw / 2., end = ls + hw / 2.;
            long aa = (long)ceil((beg - begin_wave) / mask_step);
            long bb = (long)(ceil((end - begin_wave) / mask_step) - 1);
            if (aa - 1 < 0 || bb + 1 >= n_ext || aa >= n_ext || bb < 0) { rc = -1; break; }
            double fsb = we[aa] - we[aa - 1];
            double fsa = we[bb + 1] - we[bb];
            double frb = fabs(we[aa] - beg) / fsb;
            double fra = fabs(we[bb] - end) / fsa;
            double w = line_weight[l];
            for (long k = aa; k < bb; k++) mask[k] = w;
            mask[aa - 1] = w * frb;
            mask[bb] = w * fra;
        }
        for (int j = 0; j < n_w; j++) M[(size_t)iv * n_w + j] = mask[index_old + j];
    }
    free(mask);
    free(we);
    return rc;
}

/* a16: CCF_func.py:27-36 calculate_CCF_2 (plain sequential sums) */
void orc_ccf(int n_v, int n_w, const double *M, const double *spec, double *ccf)
{
    for (int iv = 0; iv < n_v; iv++) {
        double acc = 0.0;
        const double *row = M + (size_t)iv * n_w;
        for (int j = 0; j < n_w; j++) acc += spec[j] * row[j];
        ccf[iv] = acc;
    }
}

/* run_all_SOAP.py:306-314,369-370: normalise by max, cosine apodisation */
void orc_ccf_normalise(int n_v, double *ccf)
{
    double mx = ccf[0];
    for (int i = 1; i < n_v; i++) if (ccf[i] > mx) mx = ccf[i];
    int nb_zeros = 5;
    int period = (int)((n_v - 1) / 2.);
    int len_app = (int)(period / 2.);
    int n_ones = n_v - period - 2 * nb_zeros;
    for (int i = 0; i < n_v; i++) {
        double app;
        if (i < nb_zeros) app = 0.0;
        else if (i < nb_zeros + len_app) { int a = i - nb_zeros; app = 0.5 * cos(2 * PI_REF / period * a - PI_REF) + 0.5; }
        else if (i < nb_zeros + len_app + n_ones) app = 1.0;
        else if (i < nb_zeros + 2 * len_app + n_ones) { int a = len_app - 1 - (i - nb_zeros - len_app - n_ones); app = 0.5 * cos(2 * PI_REF / period * a - PI_REF) + 0.5; }
        else app = 0.0;
        double v = ccf[i] / mx;
        ccf[i] = 1 - ((-v + 1) * app);
    }
}

/* ------------------------------------------------------------------------- */
/* a17-a18: Gaussian fit + bisector (BIS_FIT2.cpp:31-81,97-317).             */
/* The fit restates GSL's trust-region Levenberg-Marquardt with More scaling  */
/* and Nielsen's damping update (GSL >= 2.0 multifit_nlinear defaults), with   */
/* xtol = gtol = 1e-8, ftol = 0, max_iter = 10000 (BIS_FIT2.cpp:128-131).       */
/* par: [c, |k|, span, v0, fwhm]; depth/bis: 91 each; model: n                 */
/* ------------------------------------------------------------------------- */
static void orc_gauss_model(int n, const double *x, const double *p, double *fit)
{
    double sigma = p[3] / 2 / sqrt(2 * log(2));
    for (int i = 0; i < n; i++)
        fit[i] = p[0] + p[1] * exp(-(x[i] - p[2]) * (x[i] - p[2]) / 2 / sigma / sigma);
}

static void orc_gauss_jac(int n, const double *x, const double *err, const double *p, double *J)
{
    double k = p[1], x0 = p[2];
    double sigma = p[3] / 2 / sqrt(2 * log(2));
    for (int i = 0; i < n; i++) {
        double e = exp(-(x[i] - x0) * (x[i] - x0) / 2 / sigma / sigma);
        J[i * 4 + 0] = 1 / err[i];
        J[i * 4 + 1] = e / err[i];
        J[i * 4 + 2] = k / err[i] * e * (x[i] - x0) / sigma / sigma;
        J[i * 4 + 3] = k / err[i] * e * (x[i] - x0) * (x[i] - x0) / sigma / sigma / sigma / 2 / sqrt(2 * log(2));
    }
}

/* solve (A) x = b for a symmetric positive definite 4x4 via Cholesky; 0 = ok */
static int orc_chol4(const double A[16], const double b[4], double x[4])
{
    double L[16] = {0};
    for (int i = 0; i < 4; i++) {
        for (int j = 0; j <= i; j++) {
            double s = A[i * 4 + j];
            for (int k = 0; k < j; k++) s -= L[i * 4 + k] * L[j * 4 + k];
            if (i == j) { if (!(s > 0)) return -1; L[i * 4 + i] = sqrt(s); }
            else L[i * 4 + j] = s / L[j * 4 + j];
        }
    }
    double y[4];
    for (int i = 0; i < 4; i++) { double s = b[i]; for (int k = 0; k < i; k++) s -= L[i * 4 + k] * y[k]; y[i] = s / L[i * 4 + i]; }
    for (int i = 3; i >= 0; i--) { double s = y[i]; for (int k = i + 1; k < 4; k++) s -= L[k * 4 + i] * x[k]; x[i] = s / L[i * 4 + i]; }
    return 0;
}

/* returns number of iterations (>= 0) or -1 on failure */
int orc_gauss_fit(int n, const double *xr, const double *y, const double *err, double *p)
{
    double *fit = (double *)malloc(sizeof(double) * n);
    double *f = (double *)malloc(sizeof(double) * n);
    double *ft = (double *)malloc(sizeof(double) * n);
    double *J = (double *)malloc(sizeof(double) * n * 4);
    double D[4], x[4], xt[4];
    for (int q = 0; q < 4; q++) x[q] = p[q];
    orc_gauss_model(n, xr, x, fit);
    for (int i = 0; i < n; i++) f[i] = (fit[i] - y[i]) / err[i];
    orc_gauss_jac(n, xr, err, x, J);
    double JtJ[16], g[4];
    for (int a = 0; a < 4; a++) { D[a] = 0; }
    for (int i = 0; i < n; i++) for (int a = 0; a < 4; a++) D[a] += J[i * 4 + a] * J[i * 4 + a];
    for (int a = 0; a < 4; a++) D[a] = sqrt(D[a]);
    for (int a = 0; a < 4; a++) if (D[a] == 0.0) D[a] = 1.0;   /* More scaling init */
    /* Nielsen initialisation: mu = 1e-3 * max_j (||J_j|| / D_j)^2 */
    double mu = 0.0, nu = 2.0;
    for (int a = 0; a < 4; a++) {
        double cn = 0; for (int i = 0; i < n; i++) cn += J[i * 4 + a] * J[i * 4 + a];
        double t = sqrt(cn) / D[a]; if (t * t > mu) mu = t * t;
    }
    mu *= 1e-3;
    int iter = 0, status = -1;
    const double xtol = 1e-8, gtol = 1e-8;
    for (iter = 1; iter <= 10000; iter++) {
        for (int a = 0; a < 16; a++) JtJ[a] = 0;
        for (int a = 0; a < 4; a++) g[a] = 0;
        for (int i = 0; i < n; i++)
            for (int a = 0; a < 4; a++) {
                g[a] += J[i * 4 + a] * f[i];
                for (int b2 = 0; b2 < 4; b2++) JtJ[a * 4 + b2] += J[i * 4 + a] * J[i * 4 + b2];
            }
        double phi = 0; for (int i = 0; i < n; i++) phi += f[i] * f[i];
        int accepted = 0, bad = 0;
        double dx[4];
        while (!accepted) {
            double A[16], rhs[4];
            for (int a = 0; a < 16; a++) A[a] = JtJ[a];
            for (int a = 0; a < 4; a++) { A[a * 4 + a] += mu * D[a] * D[a]; rhs[a] = -g[a]; }
            if (orc_chol4(A, rhs, dx) != 0) { mu *= nu; nu *= 2; if (++bad > 15) break; continue; }
            for (int a = 0; a < 4; a++) xt[a] = x[a] + dx[a];
            orc_gauss_model(n, xr, xt, fit);
            double phit = 0;
            for (int i = 0; i < n; i++) { ft[i] = (fit[i] - y[i]) / err[i]; phit += ft[i] * ft[i]; }
            /* predicted reduction of the linear model */
            double Jdx_sq = 0, pred;
            for (int i = 0; i < n; i++) { double s = 0; for (int a = 0; a < 4; a++) s += J[i * 4 + a] * dx[a]; Jdx_sq += s * s; }
            double mud = 0; for (int a = 0; a < 4; a++) mud += mu * D[a] * D[a] * dx[a] * dx[a];
            pred = Jdx_sq + 2 * mud;
            double rho = (pred > 0) ? (phi - phit) / pred : -1.0;
            if (rho > 0) {
                accepted = 1;
                double t = 2 * rho - 1; double fac = 1 - t * t * t; if (fac < 1.0 / 3.0) fac = 1.0 / 3.0;
                mu *= fac; nu = 2;
                for (int a = 0; a < 4; a++) x[a] = xt[a];
                for (int i = 0; i < n; i++) f[i] = ft[i];
                orc_gauss_jac(n, xr, err, x, J);
                for (int a = 0; a < 4; a++) { double cn = 0; for (int i = 0; i < n; i++) cn += J[i * 4 + a] * J[i * 4 + a]; cn = sqrt(cn); if (cn > D[a]) D[a] = cn; }
            } else {
                mu *= nu; nu *= 2;
                if (++bad > 15) break;
            }
        }
        if (!accepted) {
            /* no acceptable step: converged if the last (rejected) step already meets
             * the tolerances (GSL's driver tests after ENOPROG) */
            int xok = 1;
            for (int a = 0; a < 4; a++) if (fabs(dx[a]) > xtol * (fabs(x[a]) + xtol)) xok = 0;
            double gn = 0;
            for (int a = 0; a < 4; a++) {
                double xs = fabs(x[a]) > 1.0 ? fabs(x[a]) : 1.0;
                double t = fabs(g[a] * xs); if (t > gn) gn = t;
            }
            status = (xok || gn <= gtol * (0.5 * phi > 1.0 ? 0.5 * phi : 1.0)) ? iter : -1;
            break;
        }
        /* convergence tests (GSL multifit_nlinear_test): xtol on the step, gtol on
         * the scaled gradient */
        int xok = 1;
        for (int a = 0; a < 4; a++) if (fabs(dx[a]) > xtol * (fabs(x[a]) + xtol)) xok = 0;
        double gn = 0; double phin = 0;
        for (int i = 0; i < n; i++) phin += f[i] * f[i];
        for (int a = 0; a < 4; a++) {
            double ga = 0; for (int i = 0; i < n; i++) ga += J[i * 4 + a] * f[i];
            double xs = fabs(x[a]) > 1.0 ? fabs(x[a]) : 1.0;
            double t = fabs(ga * xs); if (t > gn) gn = t;
        }
        double fmax = 0.5 * phin > 1.0 ? 0.5 * phin : 1.0;
        if (xok || gn <= gtol * fmax) { status = iter; break; }
    }
    for (int q = 0; q < 4; q++) p[q] = x[q];
    free(fit); free(f); free(ft); free(J);
    return status;
}

int orc_gauss_bis(int n, const double *xin, const double *y, const double *err,
                  double *model, double *par, double *depth_out, double *bis_out)
{
    double *x = (double *)malloc(sizeof(double) * n);
    for (int i = 0; i < n; i++) x[i] = xin[i] - xin[0];          /* BIS_FIT2.cpp:152-153 */
    double c = (y[0] + y[n - 1]) / 2;                              /* :155-160 */
    double fwhm = (x[n - 1] - x[0]) / 5.;
    double k = 0., x0 = x[n / 2];
    for (int i = 0; i < n; i++)
        if (fabs(y[i] - c) > fabs(k)) { k = y[i] - c; x0 = x[i]; }
    double p[4] = {c, k, x0, fwhm};
    int it = orc_gauss_fit(n, x, y, err, p);
    c = p[0]; k = p[1]; x0 = p[2]; fwhm = p[3];
    orc_gauss_model(n, x, p, model);
    /* bisector, BIS_FIT2.cpp:214-268 */
    int nstep = 100, margin = 5, len_depth = nstep - 2 * margin + 1;
    double sigma = fwhm / 2. / pow(2. * log(2.), .5), v0 = x0 + xin[0];
    double *norm = (double *)malloc(sizeof(double) * n);
    double *p0 = (double *)calloc(n, sizeof(double));
    double *p1 = (double *)calloc(n, sizeof(double));
    double *p2 = (double *)calloc(n, sizeof(double));
    double depth[128], bis[128];
    for (int i = 0; i < n; i++) norm[i] = -c / k * (1. - y[i] / c);
    for (int i = 0; i < len_depth; i++) depth[i] = (double)(i + margin) / nstep;
    for (int i = 0; i < n - 1; i++) {
        double vr = (xin[i] + xin[i + 1]) / 2.;
        double dd = vr - v0;
        double dC = -dd / (sigma * sigma) * exp(-(dd * dd) / 2. / (sigma * sigma));
        double d2C = ((dd * dd) / (sigma * sigma) - 1) / (sigma * sigma) * exp(-(dd * dd) / 2. / (sigma * sigma));
        double d2R = -d2C / (dC * dC * dC);
        p2[i] = d2R / 2.;
        p1[i] = (xin[i + 1] - xin[i] - p2[i] * (norm[i + 1] * norm[i + 1] - norm[i] * norm[i])) / (norm[i + 1] - norm[i]);
        p0[i] = xin[i] - p1[i] * norm[i] - p2[i] * (norm[i] * norm[i]);
    }
    int ind_max = 0;
    for (int i = 0; i < n; i++) if (norm[i] > norm[ind_max]) ind_max = i;
    for (int i = 0; i < len_depth; i++) {
        int i_b = ind_max, i_r = ind_max;
        while ((norm[i_b] > depth[i]) && (i_b > 1)) i_b--;
        while ((norm[i_r + 1] > depth[i]) && (i_r < (n - 2))) i_r++;
        bis[i] = (p0[i_b] + p0[i_r]) + (p1[i_b] + p1[i_r]) * depth[i] + (p2[i_b] + p2[i_r]) * (depth[i] * depth[i]);
        bis[i] /= 2.;
    }
    int n1 = 0, n2 = 0;
    double top = 0., bottom = 0.;
    for (int i = 0; i < len_depth; i++) {
        if ((depth[i] >= 0.1) && (depth[i] <= 0.4)) { n1++; top += bis[i]; }
        if ((depth[i] >= 0.6) && (depth[i] <= 0.9)) { n2++; bottom += bis[i]; }
    }
    top /= n1; bottom /= n2;
    par[0] = c; par[1] = fabs(k); par[2] = top - bottom; par[3] = v0; par[4] = fwhm;
    for (int i = 0; i < len_depth; i++) { depth_out[i] = 1.0 - fabs(k) * depth[i]; bis_out[i] = bis[i]; }
    free(x); free(norm); free(p0); free(p1); free(p2);
    return it;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
