// a17-a18: Gaussian fit of the CCF and its bisector, batched.
//
// Reference: BIS_FIT2.cpp:31-81 (model and analytic Jacobian), :97-192 (GSL
// multifit_nlinear trust region with default parameters: Levenberg-Marquardt,
// More scaling, xtol = gtol = 1e-8, ftol = 0, max_iter = 10000) and :214-317
// (bisector on 91 depths, span).  The reference spawns one BIS_FIT2 process per
// spectrum and exchanges text files with it.  Here one warp fits one spectrum:
// the lanes evaluate residuals and Jacobian rows, warp shuffles reduce J^T J and
// J^T f, and every lane solves the 4x4 damped normal equations redundantly (no
// divergence, no shared state).  Damping follows Nielsen's rule as in GSL
// (mu *= max(1/3, 1-(2 rho-1)^3) on acceptance, mu *= nu, nu *= 2 on rejection).
// All iteration loops are bounded.
#include <cmath>

#include "internal.cuh"

using namespace soapgb;

#define FIT_WARPS 4
#define FIT_DEPTHS 91

// butterfly sum; the final broadcast makes every lane hold lane 0's bits, so all
// lanes take identical branches in the iteration below
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return __shfl_sync(0xffffffffu, v, 0);
}

__device__ __forceinline__ double gauss_sigma(double fwhm) { return fwhm / 2 / sqrt(2 * log(2.0)); }

// solve (A) x = b (4x4 SPD) by Cholesky; returns false if not positive definite
__device__ bool chol4(const double *A, const double *b, double *x) {
    double L[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) L[q] = 0.0;
    for (int i = 0; i < 4; i++) {
        for (int j = 0; j <= i; j++) {
            double s = A[i * 4 + j];
            for (int k = 0; k < j; k++) s -= L[i * 4 + k] * L[j * 4 + k];
            if (i == j) {
                if (!(s > 0)) return false;
                L[i * 4 + i] = sqrt(s);
            } else {
                L[i * 4 + j] = s / L[j * 4 + j];
            }
        }
    }
    double y[4];
    for (int i = 0; i < 4; i++) {
        double s = b[i];
        for (int k = 0; k < i; k++) s -= L[i * 4 + k] * y[k];
        y[i] = s / L[i * 4 + i];
    }
    for (int i = 3; i >= 0; i--) {
        double s = y[i];
        for (int k = i + 1; k < 4; k++) s -= L[k * 4 + i] * x[k];
        x[i] = s / L[i * 4 + i];
    }
    return true;
}

// residual sum of squares at parameters p (lane-partial sums reduced)
__device__ double lane_phi(int n, const double *__restrict__ x, const double *__restrict__ y,
                           const double *__restrict__ err, const double *p, int lane) {
    double sigma = gauss_sigma(p[3]);
    double acc = 0.0;
    for (int i = lane; i < n; i += 32) {
        double d = x[i] - p[2];
        double fit = p[0] + p[1] * exp(-d * d / 2 / sigma / sigma);
        double f = (fit - y[i]) / (err ? err[i] : 1.0);
        acc += f * f;
    }
    return warp_sum(acc);
}

__global__ void __launch_bounds__(32 * FIT_WARPS) k_gauss_bis(int n_spec, int n, const double *__restrict__ xin,
                                                              const double *__restrict__ yall,
                                                              const double *__restrict__ errall,
                                                              double *__restrict__ xr_scr, double *__restrict__ model,
                                                              double *__restrict__ par, double *__restrict__ depth_out,
                                                              double *__restrict__ bis_out, int *__restrict__ iters,
                                                              double *__restrict__ scratch) {
    int lane = threadIdx.x & 31;
    int s = blockIdx.x * FIT_WARPS + (threadIdx.x >> 5);
    if (s >= n_spec) return;
    const double *y = yall + (long long)s * n;
    const double *err = errall ? errall + (long long)s * n : nullptr;
    const double *x = xr_scr;   // rebased velocities x - x[0] (shared by all spectra)
    // initial guess, BIS_FIT2.cpp:155-160 (done by every lane, identical)
    double c = (y[0] + y[n - 1]) / 2;
    double fwhm = (x[n - 1] - x[0]) / 5.;
    double k = 0., x0 = x[n / 2];
    for (int i = 0; i < n; i++)
        if (fabs(y[i] - c) > fabs(k)) { k = y[i] - c; x0 = x[i]; }
    double p[4] = {c, k, x0, fwhm};
    double D[4] = {0, 0, 0, 0};
    double mu = 0.0, nu = 2.0;
    double dx[4] = {0, 0, 0, 0};
    int status = -1;
    const double xtol = 1e-8, gtol = 1e-8;
    for (int iter = 0; iter <= 10000; ++iter) {
        // J^T J, J^T f, phi at p
        double sigma = gauss_sigma(p[3]);
        double jtj[10], g[4], phi = 0.0;
#pragma unroll
        for (int q = 0; q < 10; ++q) jtj[q] = 0.0;
#pragma unroll
        for (int q = 0; q < 4; ++q) g[q] = 0.0;
        for (int i = lane; i < n; i += 32) {
            double inv = 1.0 / (err ? err[i] : 1.0);
            double d = x[i] - p[2];
            double e = exp(-d * d / 2 / sigma / sigma);
            double f = (p[0] + p[1] * e - y[i]) * inv;
            double J[4];
            J[0] = inv;
            J[1] = e * inv;
            J[2] = p[1] * inv * e * d / sigma / sigma;
            J[3] = p[1] * inv * e * d * d / sigma / sigma / sigma / 2 / sqrt(2 * log(2.0));
            int t = 0;
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                g[a] += J[a] * f;
#pragma unroll
                for (int b = a; b < 4; ++b) jtj[t++] += J[a] * J[b];
            }
            phi += f * f;
        }
#pragma unroll
        for (int q = 0; q < 10; ++q) jtj[q] = warp_sum(jtj[q]);
#pragma unroll
        for (int q = 0; q < 4; ++q) g[q] = warp_sum(g[q]);
        phi = warp_sum(phi);
        double A[16];
        {
            int t = 0;
            for (int a = 0; a < 4; ++a)
                for (int b = a; b < 4; ++b) { A[a * 4 + b] = jtj[t]; A[b * 4 + a] = jtj[t]; ++t; }
        }
        if (iter == 0) {
            for (int a = 0; a < 4; ++a) { D[a] = sqrt(A[a * 5]); if (D[a] == 0.0) D[a] = 1.0; }
            double mx = 0.0;
            for (int a = 0; a < 4; ++a) { double t = sqrt(A[a * 5]) / D[a]; mx = fmax(mx, t * t); }
            mu = 1e-3 * mx;
        } else {
            for (int a = 0; a < 4; ++a) D[a] = fmax(D[a], sqrt(A[a * 5]));
            // convergence tests after an accepted step (GSL multifit_nlinear_test)
            bool xok = true;
            for (int a = 0; a < 4; ++a)
                if (fabs(dx[a]) > xtol * (fabs(p[a]) + xtol)) xok = false;
            double gn = 0.0;
            for (int a = 0; a < 4; ++a) gn = fmax(gn, fabs(g[a] * fmax(fabs(p[a]), 1.0)));
            if (xok || gn <= gtol * fmax(0.5 * phi, 1.0)) { status = iter; break; }
            if (iter == 10000) break;
        }
        // inner loop: find an acceptable step (at most 16 consecutive rejections)
        bool accepted = false;
        int bad = 0;
        while (!accepted && bad <= 15) {
            double M[16], rhs[4];
            for (int q = 0; q < 16; ++q) M[q] = A[q];
            for (int a = 0; a < 4; ++a) { M[a * 5] += mu * D[a] * D[a]; rhs[a] = -g[a]; }
            if (!chol4(M, rhs, dx)) { mu *= nu; nu *= 2; ++bad; continue; }
            double pt[4];
            for (int a = 0; a < 4; ++a) pt[a] = p[a] + dx[a];
            double phit = lane_phi(n, x, y, err, pt, lane);
            double jdx = 0.0;   // ||J dx||^2 = dx^T (J^T J) dx
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 4; ++b) jdx += dx[a] * A[a * 4 + b] * dx[b];
            double mud = 0.0;
            for (int a = 0; a < 4; ++a) mud += mu * D[a] * D[a] * dx[a] * dx[a];
            double pred = jdx + 2 * mud;
            double rho = (pred > 0 && phit < phi) ? (phi - phit) / pred : -1.0;
            if (rho > 0) {
                accepted = true;
                double t = 2 * rho - 1;
                double fac = 1 - t * t * t;
                mu *= fmax(fac, 1.0 / 3.0);
                nu = 2;
                for (int a = 0; a < 4; ++a) p[a] = pt[a];
            } else {
                mu *= nu;
                nu *= 2;
                ++bad;
            }
        }
        if (!accepted) {
            // no acceptable step: converged if the last (rejected) step already
            // meets the tolerances, as GSL's driver tests it after ENOPROG
            bool xok = true;
            for (int a = 0; a < 4; ++a)
                if (fabs(dx[a]) > xtol * (fabs(p[a]) + xtol)) xok = false;
            double gn = 0.0;
            for (int a = 0; a < 4; ++a) gn = fmax(gn, fabs(g[a] * fmax(fabs(p[a]), 1.0)));
            status = (xok || gn <= gtol * fmax(0.5 * phi, 1.0)) ? iter + 1 : -1;
            break;
        }
    }
    c = p[0]; k = p[1]; x0 = p[2]; fwhm = p[3];
    double sigma = gauss_sigma(fwhm);
    for (int i = lane; i < n; i += 32) {
        double d = x[i] - x0;
        model[(long long)s * n + i] = c + k * exp(-d * d / 2 / sigma / sigma);
    }
    // bisector, BIS_FIT2.cpp:214-268
    double *norm = scratch + (long long)s * 4 * n;
    double *p0 = norm + n, *p1 = norm + 2 * n, *p2 = norm + 3 * n;
    double sig_b = fwhm / 2. / pow(2. * log(2.), .5);
    double v0 = x0 + xin[0];
    for (int i = lane; i < n; i += 32) norm[i] = -c / k * (1. - y[i] / c);
    if (lane == 0) { p0[n - 1] = 0.0; p1[n - 1] = 0.0; p2[n - 1] = 0.0; }   // never set by the loop below
    __syncwarp();
    for (int i = lane; i < n - 1; i += 32) {
        double vr = (xin[i] + xin[i + 1]) / 2.;
        double dd = vr - v0;
        double ss = sig_b * sig_b;
        double dC = -dd / ss * exp(-(dd * dd) / 2. / ss);
        double d2C = ((dd * dd) / ss - 1) / ss * exp(-(dd * dd) / 2. / ss);
        double d2R = -d2C / (dC * dC * dC);
        double q2 = d2R / 2.;
        double a0 = norm[i], a1 = norm[i + 1];
        double q1 = (xin[i + 1] - xin[i] - q2 * (a1 * a1 - a0 * a0)) / (a1 - a0);
        p2[i] = q2;
        p1[i] = q1;
        p0[i] = xin[i] - q1 * a0 - q2 * (a0 * a0);
    }
    __syncwarp();
    int ind_max = 0;
    for (int i = 0; i < n; i++) if (norm[i] > norm[ind_max]) ind_max = i;
    double *bo = bis_out + (long long)s * FIT_DEPTHS;
    for (int t = lane; t < FIT_DEPTHS; t += 32) {
        double dep = (double)(t + 5) / 100;
        int i_b = ind_max, i_r = ind_max;
        while ((norm[i_b] > dep) && (i_b > 1)) i_b--;
        while ((norm[i_r + 1] > dep) && (i_r < (n - 2))) i_r++;
        double b = (p0[i_b] + p0[i_r]) + (p1[i_b] + p1[i_r]) * dep + (p2[i_b] + p2[i_r]) * (dep * dep);
        b /= 2.;
        bo[t] = b;
        depth_out[(long long)s * FIT_DEPTHS + t] = 1.0 - fabs(k) * dep;
    }
    __syncwarp();
    if (lane == 0) {
        // span in the reference's summation order, BIS_FIT2.cpp:256-268
        double top = 0.0, bottom = 0.0;
        int n1 = 0, n2 = 0;
        for (int t = 0; t < FIT_DEPTHS; ++t) {
            double dep = (double)(t + 5) / 100;
            if ((dep >= 0.1) && (dep <= 0.4)) { n1++; top += bo[t]; }
            if ((dep >= 0.6) && (dep <= 0.9)) { n2++; bottom += bo[t]; }
        }
        top /= n1;
        bottom /= n2;
        double *pp = par + (long long)s * 5;
        pp[0] = c;
        pp[1] = fabs(k);
        pp[2] = top - bottom;
        pp[3] = v0;
        pp[4] = fwhm;
        if (iters) iters[s] = status;
    }
}

__global__ void k_rebase(int n, const double *__restrict__ x, double *xr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) xr[i] = x[i] - x[0];
}

extern "C" int soapgb_gauss_bis(soapgb_ctx *ctx, int n_spec, int n, const double *x, const double *y,
                                const double *err, int mem, double *model, double *par, double *depth, double *bis,
                                int *iters) {
    if (!ctx) return SOAPGB_ERR_ARG;
    if (n_spec < 0 || n < 8 || !x || !y || !model || !par || !depth || !bis)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_gauss_bis: bad arguments");
    if (n_spec == 0) return SOAPGB_OK;
    SOAP_DEVICE(ctx);
    bool host = (mem == SOAPGB_HOST);
    Workspace ws(ctx);
    int s_x = ws.add(host ? sizeof(double) * n : 0);
    int s_y = ws.add(host ? sizeof(double) * (size_t)n * n_spec : 0);
    int s_e = ws.add(host && err ? sizeof(double) * (size_t)n * n_spec : 0);
    int s_model = ws.add(host ? sizeof(double) * (size_t)n * n_spec : 0);
    int s_par = ws.add(host ? sizeof(double) * 5 * n_spec : 0);
    int s_dep = ws.add(host ? sizeof(double) * FIT_DEPTHS * n_spec : 0);
    int s_bis = ws.add(host ? sizeof(double) * FIT_DEPTHS * n_spec : 0);
    int s_it = ws.add(host && iters ? sizeof(int) * n_spec : 0);
    int s_xr = ws.add(sizeof(double) * n);
    int s_scr = ws.add(sizeof(double) * 4 * (size_t)n * n_spec);
    int rc = ws.commit();
    if (rc) return rc;
    const double *d_x = (const double *)stage_in(ctx, mem, x, sizeof(double) * n, ws.get<void>(s_x), &rc);
    if (rc) return rc;
    const double *d_y = (const double *)stage_in(ctx, mem, y, sizeof(double) * (size_t)n * n_spec, ws.get<void>(s_y), &rc);
    if (rc) return rc;
    const double *d_e = (const double *)stage_in(ctx, mem, err, err ? sizeof(double) * (size_t)n * n_spec : 0, ws.get<void>(s_e), &rc);
    if (rc) return rc;
    double *d_model = host ? ws.get<double>(s_model) : model;
    double *d_par = host ? ws.get<double>(s_par) : par;
    double *d_dep = host ? ws.get<double>(s_dep) : depth;
    double *d_bis = host ? ws.get<double>(s_bis) : bis;
    int *d_it = iters ? (host ? ws.get<int>(s_it) : iters) : nullptr;
    double *xr = ws.get<double>(s_xr);
    k_rebase<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, d_x, xr);
    SOAP_LAUNCHED(ctx);
    SOAP_TRACED(ctx, "gauss_bis", k_gauss_bis<<<(n_spec + FIT_WARPS - 1) / FIT_WARPS, 32 * FIT_WARPS, 0, ctx->stream>>>(
        n_spec, n, d_x, d_y, d_e, xr, d_model, d_par, d_dep, d_bis, d_it, ws.get<double>(s_scr)));
    SOAP_LAUNCHED(ctx);
    if (host) {
        SOAP_CUDA(ctx, cudaMemcpyAsync(model, d_model, sizeof(double) * (size_t)n * n_spec, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(par, d_par, sizeof(double) * 5 * n_spec, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(depth, d_dep, sizeof(double) * FIT_DEPTHS * n_spec, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(bis, d_bis, sizeof(double) * FIT_DEPTHS * n_spec, cudaMemcpyDeviceToHost, ctx->stream));
        if (iters) SOAP_CUDA(ctx, cudaMemcpyAsync(iters, d_it, sizeof(int) * n_spec, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return host ? check_status(ctx, "soapgb_gauss_bis") : SOAPGB_OK;
}

// ---------------------------------------------------------------------------
// Adjoint of the Gaussian fit (the differentiable form; the reference has no
// gradient path).  At the fitted optimum theta = (c, k, x0, fwhm) of
// Phi = sum_i f_i^2, f_i = (G(x_i; theta) - y_i) / err_i, the stationarity condition
// sum_i f_i df_i/dtheta = 0 gives, by the implicit function theorem,
//   H dtheta/dy_j = grad G_j / err_j^2,   H = sum_i (J_i J_i^T + f_i Hess f_i)
// so dL/dy_j = (grad G_j . z) / err_j^2 with H z = dL/dtheta.  The second derivatives
// of G = c + k e, e = exp(-d^2 / 2 s^2), d = x - x0, s = a fwhm, a = 1 / (2 sqrt(2 ln 2)):
//   G_k,x0 = e d / s^2          G_k,fwhm = a e d^2 / s^3
//   G_x0,x0 = k e (d^2 / s^4 - 1 / s^2)
//   G_x0,fwhm = a k e d (d^2 / s^5 - 2 / s^3)
//   G_fwhm,fwhm = a^2 k e d^2 (d^2 / s^6 - 3 / s^4)   (all c terms vanish).
// The fitted outputs give c, |k|, v0 = x0 + x[0] and fwhm; the sign of k is that of
// the model's largest excursion from c.  One warp per spectrum, fixed reduction order.
// ---------------------------------------------------------------------------
// 4x4 solve by Gaussian elimination with partial pivoting; false when singular
__device__ bool solve4(double *A, double *b, double *z) {
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if (fabs(A[r * 4 + c]) > fabs(A[piv * 4 + c])) piv = r;
        if (!(fabs(A[piv * 4 + c]) > 0.0)) return false;
        if (piv != c) {
            for (int q = 0; q < 4; ++q) { double t = A[c * 4 + q]; A[c * 4 + q] = A[piv * 4 + q]; A[piv * 4 + q] = t; }
            double t = b[c]; b[c] = b[piv]; b[piv] = t;
        }
        for (int r = c + 1; r < 4; ++r) {
            double f = A[r * 4 + c] / A[c * 4 + c];
            for (int q = c; q < 4; ++q) A[r * 4 + q] -= f * A[c * 4 + q];
            b[r] -= f * b[c];
        }
    }
    for (int r = 3; r >= 0; --r) {
        double t = b[r];
        for (int q = r + 1; q < 4; ++q) t -= A[r * 4 + q] * z[q];
        z[r] = t / A[r * 4 + r];
    }
    return true;
}

__global__ void __launch_bounds__(32 * FIT_WARPS) k_gauss_fit_adj(int n_spec, int n, const double *__restrict__ x,
                                                                  const double *__restrict__ yall,
                                                                  const double *__restrict__ errall,
                                                                  const double *__restrict__ model,
                                                                  const double *__restrict__ par,
                                                                  const double *__restrict__ gpar,
                                                                  double *__restrict__ grad_y, int *status) {
    const int lane = threadIdx.x & 31;
    const int s = blockIdx.x * FIT_WARPS + (threadIdx.x >> 5);
    if (s >= n_spec) return;
    const double *y = yall + (long long)s * n;
    const double *err = errall ? errall + (long long)s * n : nullptr;
    const double *mo = model + (long long)s * n;
    const double *pp = par + (long long)s * 5;
    const double *gp = gpar + (long long)s * 5;
    double *gy = grad_y + (long long)s * n;
    const double c = pp[0], v0 = pp[3], fwhm = pp[4];
    // sign of k: the model's largest excursion from c (first index at ties)
    double best = -1.0, sgn = 1.0;
    int bi = n;
    for (int i = lane; i < n; i += 32) {
        const double e = fabs(mo[i] - c);
        if (e > best) { best = e; bi = i; sgn = (mo[i] - c) >= 0.0 ? 1.0 : -1.0; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        const double os = __shfl_xor_sync(0xffffffffu, sgn, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; sgn = os; }
    }
    const double k = sgn * pp[1];
    const double a = gauss_sigma(1.0);
    const double sg = gauss_sigma(fwhm);
    const double s2 = sg * sg, s3 = s2 * sg, s4 = s2 * s2;
    double H[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) H[q] = 0.0;
    for (int i = lane; i < n; i += 32) {
        const double inv = 1.0 / (err ? err[i] : 1.0);
        const double d = x[i] - v0, d2 = d * d;
        const double e = exp(-d2 / 2 / s2);
        const double f = (c + k * e - y[i]) * inv;
        const double G[4] = {1.0, e, k * e * d / s2, k * e * d2 * a / s3};
        double S[10];   // second derivatives, upper triangle row-major
        S[0] = 0.0; S[1] = 0.0; S[2] = 0.0; S[3] = 0.0;
        S[4] = 0.0;
        S[5] = e * d / s2;
        S[6] = a * e * d2 / s3;
        S[7] = k * e * (d2 / s4 - 1.0 / s2);
        S[8] = a * k * e * d * (d2 / (s4 * sg) - 2.0 / s3);
        S[9] = a * a * k * e * d2 * (d2 / (s4 * s2) - 3.0 / s4);
        int t = 0;
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int q = p; q < 4; ++q, ++t) H[t] += inv * inv * G[p] * G[q] + f * inv * S[t];
    }
#pragma unroll
    for (int q = 0; q < 10; ++q) H[q] = warp_sum(H[q]);
    double A[16], b[4] = {gp[0], gp[1] * sgn, gp[3], gp[4]}, z[4] = {0, 0, 0, 0};
    // --- the bisector span (BIS_FIT2.cpp:214-268).  Per depth the forward picks the
    // intervals i_b, i_r where the normalised CCF a_i = (y_i - c) / k crosses it (held fixed
    // here: a discrete choice) and evaluates on each the quadratic inverse
    //   P_i(d) = x_i + dx_i (d - a_i) / (a_{i+1} - a_i) + q2_i (d - a_i)(d - a_{i+1}),
    // the closed form of its p0 + p1 d + p2 d^2, with q2_i = -C''/(2 C'^3) of the fitted
    // Gaussian at the interval's middle.  The span is the mean of the bisector over depths
    // 0.1-0.4 minus its mean over 0.6-0.9; its gradient reaches y directly (a_i) and through
    // the fit's parameters (c, k in a_i; v0, sigma in q2_i), the latter added to b.
    const int wp = threadIdx.x >> 5;
    __shared__ int sp_ib[FIT_WARPS][FIT_DEPTHS], sp_ir[FIT_WARPS][FIT_DEPTHS];
    __shared__ double sp_d[FIT_WARPS][FIT_DEPTHS][4];
    const double gs = gp[2];
    if (gs != 0.0) {   // uniform for the warp
        auto nrm = [&](int i) { return -c / k * (1. - y[i] / c); };   // the forward's expression
        double bv = -1e308;
        int bix = n;
        for (int i = lane; i < n; i += 32) {
            const double v = nrm(i);
            if (v > bv) { bv = v; bix = i; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bix, o);
            if (ov > bv || (ov == bv && oi < bix)) { bv = ov; bix = oi; }
        }
        const int ind_max = bix;
        int n1 = 0, n2 = 0;
        for (int t = 0; t < FIT_DEPTHS; ++t) {
            const double dep = (double)(t + 5) / 100;
            if ((dep >= 0.1) && (dep <= 0.4)) n1++;
            if ((dep >= 0.6) && (dep <= 0.9)) n2++;
        }
        const double sig_b = fwhm / 2. / pow(2. * log(2.), .5), ss = sig_b * sig_b;
        double acc[4] = {0.0, 0.0, 0.0, 0.0};   // d span / d (c, k, v0, ss)
        for (int t = lane; t < FIT_DEPTHS; t += 32) {
            const double dep = (double)(t + 5) / 100;
            double w = 0.0;
            if ((dep >= 0.1) && (dep <= 0.4)) w += 1.0 / n1;
            if ((dep >= 0.6) && (dep <= 0.9)) w -= 1.0 / n2;
            int i_b = ind_max, i_r = ind_max;
            while ((nrm(i_b) > dep) && (i_b > 1)) i_b--;
            while ((nrm(i_r + 1) > dep) && (i_r < (n - 2))) i_r++;
            sp_ib[wp][t] = i_b;
            sp_ir[wp][t] = i_r;
            for (int side = 0; side < 2; ++side) {
                const int i = side ? i_r : i_b;
                const double a0 = nrm(i), a1 = nrm(i + 1), dx = x[i + 1] - x[i], den = a1 - a0;
                const double dd = (x[i] + x[i + 1]) / 2. - v0;
                const double e = exp(-(dd * dd) / 2. / ss);
                const double dC = -dd / ss * e, d2C = ((dd * dd) / ss - 1) / ss * e;
                const double q2 = -d2C / (2. * dC * dC * dC);
                const double d3C = e * dd * (3. - dd * dd / ss) / (ss * ss);
                const double dCs = dd * e / (ss * ss) * (1. - dd * dd / (2. * ss));
                const double d2Cs = e * ((-2. * dd * dd / (ss * ss * ss) + 1. / (ss * ss)) +
                                         (dd * dd / (ss * ss) - 1. / ss) * (dd * dd / (2. * ss * ss)));
                const double c3 = dC * dC * dC, c4 = c3 * dC;
                const double q2_dd = -0.5 * (d3C / c3 - 3. * d2C * d2C / c4);
                const double q2_ss = -0.5 * (d2Cs / c3 - 3. * d2C * dCs / c4);
                const double h = 0.5 * w;
                const double pa0 = h * (dx * (dep - a1) / (den * den) - q2 * (dep - a1));
                const double pa1 = h * (-dx * (dep - a0) / (den * den) - q2 * (dep - a0));
                const double pq2 = h * (dep - a0) * (dep - a1);
                sp_d[wp][t][2 * side] = pa0;
                sp_d[wp][t][2 * side + 1] = pa1;
                acc[0] += -(pa0 + pa1) / k;
                acc[1] += -(pa0 * a0 + pa1 * a1) / k;
                acc[2] += -pq2 * q2_dd;   // dd = vr - v0
                acc[3] += pq2 * q2_ss;
            }
        }
        b[0] += gs * warp_sum(acc[0]);
        b[1] += gs * warp_sum(acc[1]);
        b[2] += gs * warp_sum(acc[2]);
        b[3] += gs * warp_sum(acc[3]) * 2. * ss / fwhm;   // ss = (fwhm / 2 sqrt(2 ln 2))^2
    }
    __syncwarp();
    {
        int t = 0;
        for (int p = 0; p < 4; ++p)
            for (int q = p; q < 4; ++q, ++t) { A[p * 4 + q] = H[t]; A[q * 4 + p] = H[t]; }
    }
    if (!solve4(A, b, z)) {
        if (lane == 0) atomicExch(status, SOAPGB_ST_FIT_SINGULAR);
        for (int q = 0; q < 4; ++q) z[q] = 0.0;
    }
    for (int i = lane; i < n; i += 32) {
        const double inv = 1.0 / (err ? err[i] : 1.0);
        const double d = x[i] - v0, d2 = d * d;
        const double e = exp(-d2 / 2 / s2);
        double g = inv * inv * (z[0] + e * z[1] + (k * e * d / s2) * z[2] + (k * e * d2 * a / s3) * z[3]);
        if (gs != 0.0) {   // the span's direct dependence on y_i (through a_i), depths in order
            double dir = 0.0;
            for (int t = 0; t < FIT_DEPTHS; ++t) {
                const int ib = sp_ib[wp][t], ir = sp_ir[wp][t];
                if (ib == i) dir += sp_d[wp][t][0];
                if (ib + 1 == i) dir += sp_d[wp][t][1];
                if (ir == i) dir += sp_d[wp][t][2];
                if (ir + 1 == i) dir += sp_d[wp][t][3];
            }
            g += gs * dir / k;
        }
        gy[i] = g;
    }
}

extern "C" int soapgb_gauss_fit_adjoint(soapgb_ctx *ctx, int n_spec, int n, const double *x, const double *y,
                                        const double *err, const double *model, const double *par,
                                        const double *g_par, int mem, double *grad_y) {
    if (!ctx) return SOAPGB_ERR_ARG;
    if (n_spec < 0 || n < 8 || !x || !y || !model || !par || !g_par || !grad_y)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_gauss_fit_adjoint: bad arguments");
    if (n_spec == 0) return SOAPGB_OK;
    SOAP_DEVICE(ctx);
    const bool host = (mem == SOAPGB_HOST);
    const size_t sb = sizeof(double) * (size_t)n * n_spec, pb = sizeof(double) * 5 * (size_t)n_spec;
    Workspace ws(ctx);
    int s_x = ws.add(host ? sizeof(double) * n : 0);
    int s_y = ws.add(host ? sb : 0), s_e = ws.add(host && err ? sb : 0), s_m = ws.add(host ? sb : 0);
    int s_p = ws.add(host ? pb : 0), s_g = ws.add(host ? pb : 0), s_o = ws.add(host ? sb : 0);
    int rc = ws.commit();
    if (rc) return rc;
#define STAGE(dst, src, bytes, slot)                                                  \
    dst = (const double *)stage_in(ctx, mem, src, bytes, ws.get<void>(slot), &rc);   \
    if (rc) return rc;
    const double *d_x, *d_y, *d_e, *d_m, *d_p, *d_g;
    STAGE(d_x, x, sizeof(double) * n, s_x);
    STAGE(d_y, y, sb, s_y);
    STAGE(d_e, err, err ? sb : 0, s_e);
    STAGE(d_m, model, sb, s_m);
    STAGE(d_p, par, pb, s_p);
    STAGE(d_g, g_par, pb, s_g);
#undef STAGE
    double *d_o = host ? ws.get<double>(s_o) : grad_y;
    SOAP_TRACED(ctx, "gauss_fit_adjoint",
                k_gauss_fit_adj<<<(n_spec + FIT_WARPS - 1) / FIT_WARPS, 32 * FIT_WARPS, 0, ctx->stream>>>(
                    n_spec, n, d_x, d_y, d_e, d_m, d_p, d_g, d_o, ctx->d_status));
    SOAP_LAUNCHED(ctx);
    if (host) {
        SOAP_CUDA(ctx, cudaMemcpyAsync(grad_y, d_o, sb, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return check_status(ctx, "soapgb_gauss_fit_adjoint");
    }
    return SOAPGB_OK;
}
