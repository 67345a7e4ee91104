// a11-a12: per-phase active-region integration.
//
// Reference: SOAP_integration.cu:392-447 (spot_integrate: a host loop over all
// G*G cells issuing eight FP64 kernels per active cell -- shift, three
// interpolations, intensity, flux/bconv/tot) and :285-323 (the accumulation
// kernels).  Here one launch covers every phase: block (x, p) owns a pixel range
// of phase p and gathers all of the phase's active cells, in map order, into
// register accumulators.
#include <cmath>

#include "internal.cuh"
#include "fir.cuh"

using namespace soapgb;

// loi_Planck, SOAP_integration.cu:205-212
__device__ __forceinline__ double soap_planck(double lambda0, double temp) {
    double c = 299792458.;
    double h = 6.62606896e-34;
    double k_b = 1.380e-23;
    double scale = 1e-10;
    return 2 * h * pow(c, 2) * 1. / pow(lambda0 * scale, 5) * 1. / (exp((h * c) / (lambda0 * k_b * temp * scale)) - 1);
}

constexpr int PHASE_CHUNK = 256;

// One cell's interpolation geometry at pixel j (shared by the three cubes).
struct CellAt {
    long long i;   // owner source index, -1 if none
    double dd;     // l'_{i+1} - l'_i
    double dl;     // l_j - l'_i
};

__device__ __forceinline__ CellAt soap_cell_at(long long j, int n_eff, const double *__restrict__ lam,
                                               const CellShift &c) {
    CellAt r;
    r.i = soap_owner(j, n_eff, c);
    r.dd = 0.0;
    r.dl = 0.0;
    if (r.i >= 0) {
        double li = lam[r.i], li1 = lam[r.i + 1];
        double ls0 = __dadd_rn(li, __dmul_rn(__dmul_rn(-1.0, li), __dsub_rn(1.0, c.sq)));
        double ls1 = __dadd_rn(li1, __dmul_rn(__dmul_rn(-1.0, li1), __dsub_rn(1.0, c.sq)));
        r.dd = __dsub_rn(ls1, ls0);
        r.dl = __dsub_rn(lam[j], ls0);
    }
    return r;
}

__device__ __forceinline__ double soap_lerp_at(const CellAt &a, long long j, const double *__restrict__ row,
                                               double delta, double limb) {
    if (delta == 0.0) return __dmul_rn(row[j], limb);
    if (a.i < 0) return 0.0;
    double s0 = row[a.i], s1 = row[a.i + 1];
    double t = __dmul_rn(__ddiv_rn(__dsub_rn(s1, s0), a.dd), a.dl);
    return __dmul_rn(__dadd_rn(s0, t), limb);
}

__global__ void __launch_bounds__(256) k_phase_plain64(
    int n, int n_eff, const double *__restrict__ lam, const double *__restrict__ q_norm,
    const double *__restrict__ q_sed, const double *__restrict__ spot_norm, const double *__restrict__ fac_norm,
    const double *__restrict__ spot_sed, const double *__restrict__ fac_sed, int max_cells,
    const int *__restrict__ cells, const int *__restrict__ counts, const double *__restrict__ temp,
    const double *__restrict__ bi, const double *__restrict__ delta_m, const double *__restrict__ limb_m,
    const double *__restrict__ lb_m, const int *__restrict__ region_m, long long gm, double step, int solar,
    int t_star, int t_diff_fac, double *__restrict__ flux, double *__restrict__ bconv, double *__restrict__ tot,
    long long out_stride, int n_mu, int *status) {
    __shared__ double s_delta[PHASE_CHUNK], s_limb[PHASE_CHUNK], s_fb[PHASE_CHUNK], s_sq[PHASE_CHUNK],
        s_off[PHASE_CHUNK], s_lb[PHASE_CHUNK], s_temp[PHASE_CHUNK];
    __shared__ int s_row[PHASE_CHUNK], s_type[PHASE_CHUNK];
    int p = blockIdx.y;
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double lambda0 = lam[0];
    const int *pc = cells + (long long)p * max_cells;
    int nc_all = counts[p];
    const double *pt = temp + (long long)p * gm;
    const double *pb = bi + (long long)p * gm;
    double fx = 0.0, bc = 0.0, tt = 0.0;
    double lj = (j < n_eff) ? lam[j] : 0.0;
    double ssed = (j < n_eff) ? spot_sed[j] : 0.0;
    double fsed = (j < n_eff) ? fac_sed[j] : 0.0;
    int t_norm_fac = (int)(t_star + t_diff_fac + 0.9 - 216.8);
    for (int c0 = 0; c0 < nc_all; c0 += PHASE_CHUNK) {
        int nc = min(PHASE_CHUNK, nc_all - c0);
        __syncthreads();
        for (int t = threadIdx.x; t < nc; t += blockDim.x) {
            int k = pc[c0 + t];
            double d = delta_m[k];
            CellShift cs = soap_cell_shift(d, lambda0, step);
            s_delta[t] = d;
            s_limb[t] = limb_m[k];
            s_fb[t] = cs.fbeta;
            s_sq[t] = cs.sq;
            s_off[t] = cs.off;
            int row = region_m[k];
            if ((unsigned)row >= (unsigned)n_mu) {   // mu bin outside the cube: report, use bin 0
                atomicExch(status, 21);
                row = 0;
            }
            s_row[t] = row;
            s_lb[t] = lb_m[k];
            s_temp[t] = pt[k];
            s_type[t] = (pb[k] == 0.0) ? 0 : 1;
        }
        __syncthreads();
        if (j < n_eff) {
            for (int t = 0; t < nc; ++t) {
                CellShift cs;
                cs.fbeta = s_fb[t];
                cs.sq = s_sq[t];
                cs.off = s_off[t];
                double d = s_delta[t], L = s_limb[t];
                long long off = (long long)s_row[t] * n;
                CellAt at;
                if (d != 0.0) at = soap_cell_at(j, n_eff, lam, cs);
                double q = soap_lerp_at(at, j, q_norm + off, d, L);
                double s = soap_lerp_at(at, j, q_sed + off, d, L);
                double a, inten;
                if (s_type[t] == 0) {
                    // fast_intensity with T_norm = (int)T: the Planck ratio is exactly 1
                    double T = s_temp[t];
                    int tn = (int)T;
                    double ratio = ((double)tn == T) ? 1.0 : soap_planck(lj, T) / soap_planck(lj, (double)tn);
                    inten = __dmul_rn(ratio, ssed);
                    a = soap_lerp_at(at, j, spot_norm + off, d, L);
                } else {
                    if (solar) {
                        double T = s_temp[t];
                        double ratio = ((double)t_norm_fac == T) ? 1.0
                                                                  : soap_planck(lj, T) / soap_planck(lj, (double)t_norm_fac);
                        inten = __dmul_rn(ratio, fsed);
                    } else {
                        inten = __dmul_rn(__dadd_rn(1.0, s_lb[t]), fsed);
                    }
                    a = soap_lerp_at(at, j, fac_norm + off, d, L);
                }
                fx = __dsub_rn(__dadd_rn(fx, s), __dmul_rn(inten, q));
                bc = __dsub_rn(__dadd_rn(bc, q), a);
                tt = __dsub_rn(__dadd_rn(tt, s), __dmul_rn(a, inten));
            }
        }
    }
    long long o = (long long)p * out_stride + j;
    if (j < n_eff) {
        flux[o] = fx;
        bconv[o] = bc;
        tot[o] = tt;
    } else if (j < n) {
        flux[o] = 0.0;
        bconv[o] = 0.0;
        tot[o] = 0.0;
    }
}

// ---------------------------------------------------------------------------
// Adjoint of the PLAIN64 integration.  The outputs are linear in every cube row and
// in every cell's limb value L:
//   flux += s - I q,  bconv += q - a,  tot += s - I a,   q, s, a = L lerp(row)
// with lerp(row)[j] = row[o] + (row[o+1] - row[o]) (dl / dd) at the owner o of j.
// Given gF, gB, gT (gradients of a scalar w.r.t. flux, bconv, tot), the gradients
// are gathers in a fixed order (no atomics):
//   row grads: source pixel i collects from the output pixels it owns as o (weight
//     1 - dl/dd) and as o + 1 (weight dl/dd), times L and the combination of
//     gF, gB, gT the row enters with (q_sed: gF + gT; q_norm: gB - I gF;
//     spot / facula rows: -gB - I gT);
//   continuum rows: I = ratio x sed[j], so d/dsed[j] = sum over cells of
//     ratio (-q gF - a gT);
//   limb: d/dL = sum over j of the cell's unit-L contribution dotted with g;
//   velocity: the weight w = (l_j / S - l_o) / (l_{o+1} - l_o) of the owner o moves
//     with the Doppler factor S = sqrt((1 + b) / (1 - b)), b = delta 1000 / c:
//     dw/ddelta = -l_j / (S^2 (l_{o+1} - l_o)) x 1 / (S (1 - b)^2) x 1000 / c, and each
//     row's value moves by (row[o+1] - row[o]) dw/ddelta (continuous across owners).
// ---------------------------------------------------------------------------

constexpr int ADJ_MAX_MU = 256;   // mu rows the adjoint's per-phase regrouping handles

// per phase, the active cells regrouped by mu row (stable: map order within a row);
// roff[p][b .. b + 1] delimits row b.  One thread per phase (a few thousand cells).
__global__ void k_adj_bucket(int n_mu, long long gm, const int *__restrict__ cells, const int *__restrict__ counts,
                             const int *__restrict__ region_m, int *__restrict__ rcells, int *__restrict__ roff,
                             int *status) {
    __shared__ int cur[ADJ_MAX_MU + 1];
    const int p = blockIdx.x;
    if (threadIdx.x != 0) return;
    const int *pc = cells + (long long)p * gm;
    const int nc = counts[p];
    int *off = roff + (long long)p * (n_mu + 1);
    for (int b = 0; b <= n_mu; ++b) cur[b] = 0;
    for (int c = 0; c < nc; ++c) {
        int row = region_m[pc[c]];
        if ((unsigned)row >= (unsigned)n_mu) {
            atomicExch(status, 21);
            row = 0;
        }
        cur[row + 1]++;
    }
    for (int b = 1; b <= n_mu; ++b) cur[b] += cur[b - 1];
    for (int b = 0; b <= n_mu; ++b) off[b] = cur[b];
    int *pr = rcells + (long long)p * gm;
    for (int c = 0; c < nc; ++c) {
        int row = region_m[pc[c]];
        if ((unsigned)row >= (unsigned)n_mu) row = 0;
        pr[cur[row]++] = pc[c];
    }
}

// cell intensity I at pixel j (fast_intensity / fast_intensity_fac / the solar form)
__device__ __forceinline__ double soap_intensity(int type, double T, double lbk, double lj, double ssed, double fsed,
                                                 int solar, int t_norm_fac) {
    if (type == 0) {
        const int tn = (int)T;
        const double ratio = ((double)tn == T) ? 1.0 : soap_planck(lj, T) / soap_planck(lj, (double)tn);
        return __dmul_rn(ratio, ssed);
    }
    if (solar) {
        const double ratio = ((double)t_norm_fac == T) ? 1.0 : soap_planck(lj, T) / soap_planck(lj, (double)t_norm_fac);
        return __dmul_rn(ratio, fsed);
    }
    return __dmul_rn(__dadd_rn(1.0, lbk), fsed);
}

// Per-cell constants of the adjoint weights.  In exact arithmetic the shifted grid is
// l'_i = S l_i (S = sqrt((1+b)/(1-b))), so the interpolation weight of pixel j in the
// owner interval o is w = (l_j - l'_o) / (S (l_{o+1} - l_o)) and
// dw/ddelta = -l_j / (S (l_{o+1} - l_o)) * (dS/ddelta) / S, dS/ddelta = (1000/c) / (S (1-b)^2).
// With the per-interval reciprocals inv[o] = 1 / (l_{o+1} - l_o) both take multiplications
// only: w = (l_j - l'_o) * invS * inv[o], dw = -l_j * K * inv[o].  The forward rounds
// ((row[o+1] - row[o]) / (l'_{o+1} - l'_o)) (l_j - l'_o); the adjoint needs the weights, not
// that rounding (they agree to ~1e-10 of a weight).
struct AdjCell {
    CellShift cs;
    double invS;   // 1 / S (1 for v == 0)
    double K;      // (1000/c) / (S^3 (1-b)^2)
};
__device__ __forceinline__ AdjCell adj_cell(double d, double lambda0, double step) {
    AdjCell a;
    a.cs = soap_cell_shift(d, lambda0, step);
    const double beta = d * 1000. / SOAP_C_LIGHT;
    const double S = (d == 0.0) ? 1.0 : a.cs.sq;
    const double omb = 1.0 - beta;
    a.invS = 1.0 / S;
    a.K = (1000. / SOAP_C_LIGHT) / (S * S * S * omb * omb);
    return a;
}

// per-interval reciprocals inv[o] = 1 / (l_{o+1} - l_o), o < n_eff - 1
__global__ void k_adj_inv(int n_eff, const double *__restrict__ lam, double *__restrict__ inv) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o < n_eff - 1) inv[o] = 1.0 / (lam[o + 1] - lam[o]);
}

// unit-limb values of a cell's three rows at output pixel j (q_norm, q_sed and the
// spot or facula row): w at the owner o, then row[o] + (row[o+1] - row[o]) w.
struct AdjRows {
    double q, s, a;
    double dq, ds, da;   // d/ddelta of the three values (unit limb)
};
template <bool WITH_S = true>
__device__ __forceinline__ AdjRows adj_rows_at(long long j, int n_eff, const double *__restrict__ lam,
                                               const double *__restrict__ inv, const AdjCell &ac, double d,
                                               const double *__restrict__ rq, const double *__restrict__ rs,
                                               const double *__restrict__ ra) {
    AdjRows v;
    // the owner interval of j; with v == 0 the forward copies pixel j (owner j, w = 0)
    const long long o = (d == 0.0) ? ((j <= n_eff - 2) ? j : -1) : soap_owner(j, n_eff, ac.cs);
    if (o < 0) {
        v.q = (d == 0.0) ? rq[j] : 0.0;
        v.s = (d == 0.0) ? rs[j] : 0.0;
        v.a = (d == 0.0) ? ra[j] : 0.0;
        v.dq = v.ds = v.da = 0.0;
        return v;
    }
    const double lo0 = lam[o], lj = lam[j], io = inv[o];
    double w = 0.0;
    if (d != 0.0) {
        const double ls0 = __dadd_rn(lo0, __dmul_rn(__dmul_rn(-1.0, lo0), __dsub_rn(1.0, ac.cs.sq)));
        w = (lj - ls0) * ac.invS * io;
    }
    const double eq = rq[o + 1] - rq[o], es = WITH_S ? rs[o + 1] - rs[o] : 0.0, ea = ra[o + 1] - ra[o];
    v.q = fma(eq, w, rq[o]);
    v.s = WITH_S ? fma(es, w, rs[o]) : 0.0;
    v.a = fma(ea, w, ra[o]);
    const double dw = -lj * ac.K * io;
    v.dq = eq * dw;
    v.ds = es * dw;
    v.da = ea * dw;
    return v;
}

// row gradients: grid (ceil(n / 256), n_mu); thread = source pixel i of row b
// BC: the bconv gradient alone (gF = gT = 0): no intensity, no q_sed or continuum terms
template <bool BC>
__global__ void __launch_bounds__(256) k_adj_rows(
    int n, int n_eff, const double *__restrict__ lam, const double *__restrict__ inv, const double *__restrict__ spot_sed,
    const double *__restrict__ fac_sed, int n_phase, long long gm, const int *__restrict__ rcells,
    const int *__restrict__ roff, int n_mu, const double *__restrict__ temp, const double *__restrict__ bi,
    const double *__restrict__ delta_m, const double *__restrict__ limb_m, const double *__restrict__ lb_m,
    double step, int solar, int t_star, int t_diff_fac, const double *__restrict__ gF, const double *__restrict__ gB,
    const double *__restrict__ gT, long long g_stride, double *__restrict__ d_qn, double *__restrict__ d_qs,
    double *__restrict__ d_sn, double *__restrict__ d_fn) {
    __shared__ double s_delta[PHASE_CHUNK], s_limb[PHASE_CHUNK], s_fb[PHASE_CHUNK], s_sq[PHASE_CHUNK],
        s_off[PHASE_CHUNK], s_lb[PHASE_CHUNK], s_temp[PHASE_CHUNK], s_is[PHASE_CHUNK];
    __shared__ int s_type[PHASE_CHUNK];
    const int b = blockIdx.y;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const double lambda0 = lam[0];
    const int t_norm_fac = (int)(t_star + t_diff_fac + 0.9 - 216.8);
    double aqn = 0.0, aqs = 0.0, asn = 0.0, afn = 0.0;
    for (int p = 0; p < n_phase; ++p) {
        const int *off = roff + (long long)p * (n_mu + 1);
        const int c_lo = off[b], c_hi = off[b + 1];
        const int *pr = rcells + (long long)p * gm;
        const double *pt = temp + (long long)p * gm, *pb = bi + (long long)p * gm;
        const double *gf = gF + (long long)p * g_stride, *gb = gB + (long long)p * g_stride,
                     *gt = gT + (long long)p * g_stride;
        for (int c0 = c_lo; c0 < c_hi; c0 += PHASE_CHUNK) {
            const int nc = min(PHASE_CHUNK, c_hi - c0);
            __syncthreads();
            for (int t = threadIdx.x; t < nc; t += blockDim.x) {
                const int k = pr[c0 + t];
                const double d = delta_m[k];
                const CellShift cs = soap_cell_shift(d, lambda0, step);
                s_delta[t] = d;
                s_limb[t] = limb_m[k];
                s_fb[t] = cs.fbeta;
                s_sq[t] = cs.sq;
                s_off[t] = cs.off;
                s_is[t] = 1.0 / cs.sq;
                s_lb[t] = lb_m[k];
                s_temp[t] = pt[k];
                s_type[t] = (pb[k] == 0.0) ? 0 : 1;
            }
            __syncthreads();
            if (i >= n_eff) continue;
            for (int t = 0; t < nc; ++t) {
                const double L = s_limb[t];
                const int type = s_type[t];
                // contributions of output pixel j with weight w on source i
                auto add = [&](long long j, double w) {
                    const double lw = __dmul_rn(L, w);
                    if constexpr (BC) {
                        const double g = gb[j];
                        aqn = fma(lw, g, aqn);
                        if (type == 0) asn = fma(lw, -g, asn);
                        else afn = fma(lw, -g, afn);
                        return;
                    }
                    const double lj = lam[j];
                    const double I = soap_intensity(type, s_temp[t], s_lb[t], lj, spot_sed[j], fac_sed[j], solar,
                                                    t_norm_fac);
                    aqs = fma(lw, __dadd_rn(gf[j], gt[j]), aqs);
                    aqn = fma(lw, __dsub_rn(gb[j], __dmul_rn(I, gf[j])), aqn);
                    const double ha = __dsub_rn(-gb[j], __dmul_rn(I, gt[j]));
                    if (type == 0) asn = fma(lw, ha, asn);
                    else afn = fma(lw, ha, afn);
                };
                if (s_delta[t] == 0.0) {   // v == 0: output pixel i copies source i
                    add(i, 1.0);
                    continue;
                }
                CellShift cs;
                cs.fbeta = s_fb[t];
                cs.sq = s_sq[t];
                cs.off = s_off[t];
                const double invS = s_is[t];
                // owner o = i - 1 (source i is its upper neighbour) and o = i (lower); the
                // outputs of owner o are ceil(x_o) <= j < ceil(x_{o+1})
                const long long cp[3] = {soap_ceil_pos(i - 1, cs), soap_ceil_pos(i, cs), soap_ceil_pos(i + 1, cs)};
#pragma unroll
                for (int side = 0; side < 2; ++side) {
                    const long long o = i - 1 + side;
                    if (o < 0 || o > n_eff - 2) continue;
                    const long long ja = max(cp[side], 0LL);
                    const long long jb = min(cp[side + 1], (long long)n_eff);
                    if (ja >= jb) continue;
                    const double lo0 = lam[o];
                    const double ls0 = __dadd_rn(lo0, __dmul_rn(__dmul_rn(-1.0, lo0), __dsub_rn(1.0, cs.sq)));
                    const double sc = invS * inv[o];
                    for (long long j = ja; j < jb; ++j) {
                        const double r = (lam[j] - ls0) * sc;
                        add(j, side == 0 ? r : 1.0 - r);
                    }
                }
            }
        }
    }
    if (i < n) {
        const long long o = (long long)b * n + i;
        d_qn[o] = aqn;
        d_qs[o] = aqs;
        d_sn[o] = asn;
        d_fn[o] = afn;
    }
}

// continuum-row gradients: thread = output pixel j; all active cells of all phases
__global__ void __launch_bounds__(256) k_adj_continuum(
    int n, int n_eff, const double *__restrict__ lam, const double *__restrict__ inv, const double *__restrict__ q_norm,
    const double *__restrict__ spot_norm, const double *__restrict__ fac_norm, const double *__restrict__ spot_sed,
    const double *__restrict__ fac_sed, int n_phase, long long gm, const int *__restrict__ cells,
    const int *__restrict__ counts, const double *__restrict__ temp, const double *__restrict__ bi,
    const double *__restrict__ delta_m, const double *__restrict__ limb_m, const double *__restrict__ lb_m,
    const int *__restrict__ region_m, int n_mu, double step, int solar, int t_star, int t_diff_fac,
    const double *__restrict__ gF, const double *__restrict__ gT, long long g_stride, double *__restrict__ d_ss,
    double *__restrict__ d_fs) {
    __shared__ double s_delta[PHASE_CHUNK], s_limb[PHASE_CHUNK], s_fb[PHASE_CHUNK], s_sq[PHASE_CHUNK],
        s_off[PHASE_CHUNK], s_lb[PHASE_CHUNK], s_temp[PHASE_CHUNK], s_is[PHASE_CHUNK], s_k[PHASE_CHUNK];
    __shared__ int s_row[PHASE_CHUNK], s_type[PHASE_CHUNK];
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const double lambda0 = lam[0];
    const int t_norm_fac = (int)(t_star + t_diff_fac + 0.9 - 216.8);
    const double lj = (j < n_eff) ? lam[j] : 0.0;
    double ass = 0.0, afs = 0.0;
    for (int p = 0; p < n_phase; ++p) {
        const int *pc = cells + (long long)p * gm;
        const int nc_all = counts[p];
        const double *pt = temp + (long long)p * gm, *pb = bi + (long long)p * gm;
        const double gf = (j < n_eff) ? gF[(long long)p * g_stride + j] : 0.0;
        const double gt = (j < n_eff) ? gT[(long long)p * g_stride + j] : 0.0;
        for (int c0 = 0; c0 < nc_all; c0 += PHASE_CHUNK) {
            const int nc = min(PHASE_CHUNK, nc_all - c0);
            __syncthreads();
            for (int t = threadIdx.x; t < nc; t += blockDim.x) {
                const int k = pc[c0 + t];
                const double d = delta_m[k];
                const AdjCell ac = adj_cell(d, lambda0, step);
                s_delta[t] = d;
                s_limb[t] = limb_m[k];
                s_fb[t] = ac.cs.fbeta;
                s_sq[t] = ac.cs.sq;
                s_off[t] = ac.cs.off;
                s_is[t] = ac.invS;
                s_k[t] = ac.K;
                int row = region_m[k];
                s_row[t] = ((unsigned)row < (unsigned)n_mu) ? row : 0;
                s_lb[t] = lb_m[k];
                s_temp[t] = pt[k];
                s_type[t] = (pb[k] == 0.0) ? 0 : 1;
            }
            __syncthreads();
            if (j >= n_eff) continue;
            for (int t = 0; t < nc; ++t) {
                AdjCell ac;
                ac.cs.fbeta = s_fb[t];
                ac.cs.sq = s_sq[t];
                ac.cs.off = s_off[t];
                ac.invS = s_is[t];
                ac.K = s_k[t];
                const double d = s_delta[t], L = s_limb[t];
                const long long off = (long long)s_row[t] * n;
                const int type = s_type[t];
                const AdjRows v = adj_rows_at(j, n_eff, lam, inv, ac, d, q_norm + off, q_norm + off,
                                              (type == 0 ? spot_norm : fac_norm) + off);
                // d/dsed[j] of (-I q gF - I a gT) with I = ratio sed[j]; q, a carry L
                const double h = __dmul_rn(L, fma(-v.q, gf, -__dmul_rn(v.a, gt)));
                const double ratio = soap_intensity(type, s_temp[t], s_lb[t], lj, 1.0, 1.0, solar, t_norm_fac);
                if (type == 0) ass = fma(ratio, h, ass);
                else afs = fma(ratio, h, afs);
            }
        }
    }
    if (j < n) {
        d_ss[j] = ass;
        d_fs[j] = afs;
    }
}

// limb gradients per (phase, cell): block (x, p) takes the phase's cells x, x + gridDim.x,
// ...; the dot product over the pixels is reduced in a fixed order (warp shuffles,
// then warps in order) into buf[p][k]
template <bool BC>
__global__ void __launch_bounds__(256) k_adj_limb(
    int n, int n_eff, const double *__restrict__ lam, const double *__restrict__ inv, const double *__restrict__ q_norm,
    const double *__restrict__ q_sed, const double *__restrict__ spot_norm, const double *__restrict__ fac_norm,
    const double *__restrict__ spot_sed, const double *__restrict__ fac_sed, long long gm,
    const int *__restrict__ cells, const int *__restrict__ counts, const double *__restrict__ temp,
    const double *__restrict__ bi, const double *__restrict__ delta_m, const double *__restrict__ lb_m,
    const int *__restrict__ region_m, int n_mu, double step, int solar, int t_star, int t_diff_fac,
    const double *__restrict__ gF, const double *__restrict__ gB, const double *__restrict__ gT, long long g_stride,
    const double *__restrict__ limb_m, double *__restrict__ buf, double *__restrict__ buf_d) {
    __shared__ double red[2][256 / 32];
    const int p = blockIdx.y;
    const double lambda0 = lam[0];
    const int t_norm_fac = (int)(t_star + t_diff_fac + 0.9 - 216.8);
    const int *pc = cells + (long long)p * gm;
    const int nc = counts[p];
    const double *gf = gF + (long long)p * g_stride, *gb = gB + (long long)p * g_stride,
                 *gt = gT + (long long)p * g_stride;
    for (int c = blockIdx.x; c < nc; c += gridDim.x) {
        const int k = pc[c];
        const double d = delta_m[k];
        const AdjCell ac = adj_cell(d, lambda0, step);
        int row = region_m[k];
        row = ((unsigned)row < (unsigned)n_mu) ? row : 0;
        const long long off = (long long)row * n;
        const int type = (bi[(long long)p * gm + k] == 0.0) ? 0 : 1;
        const double T = temp[(long long)p * gm + k], lbk = lb_m[k];
        const double *arow = (type == 0 ? spot_norm : fac_norm) + off;
        double acc = 0.0, accd = 0.0;
        for (long long j = threadIdx.x; j < n_eff; j += blockDim.x) {
            if constexpr (BC) {   // bconv alone: (q - a) against gB
                const AdjRows v = adj_rows_at<false>(j, n_eff, lam, inv, ac, d, q_norm + off, q_norm + off, arow);
                const double g = gb[j];
                acc = fma(g, __dsub_rn(v.q, v.a), acc);
                accd = fma(g, v.dq - v.da, accd);
                continue;
            }
            const AdjRows v = adj_rows_at(j, n_eff, lam, inv, ac, d, q_norm + off, q_sed + off, arow);
            const double I = soap_intensity(type, T, lbk, lam[j], spot_sed[j], fac_sed[j], solar, t_norm_fac);
            acc = fma(gf[j], __dsub_rn(v.s, __dmul_rn(I, v.q)), acc);
            acc = fma(gb[j], __dsub_rn(v.q, v.a), acc);
            acc = fma(gt[j], __dsub_rn(v.s, __dmul_rn(I, v.a)), acc);
            accd = fma(gf[j], v.ds - I * v.dq, accd);
            accd = fma(gb[j], v.dq - v.da, accd);
            accd = fma(gt[j], v.ds - I * v.da, accd);
        }
        for (int o = 16; o > 0; o >>= 1) {
            acc += __shfl_xor_sync(0xffffffffu, acc, o);
            accd += __shfl_xor_sync(0xffffffffu, accd, o);
        }
        __syncthreads();
        if ((threadIdx.x & 31) == 0) {
            red[0][threadIdx.x >> 5] = acc;
            red[1][threadIdx.x >> 5] = accd;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double sum = 0.0, sumd = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                sum += red[0][w];
                sumd += red[1][w];
            }
            buf[(long long)p * gm + k] = sum;
            buf_d[(long long)p * gm + k] = __dmul_rn(limb_m[k], sumd);   // the values carry L
        }
    }
}

// grad_limb[k] = sum over phases, in order, of buf[p][k]
__global__ void k_adj_sum_phases(int n_phase, long long gm, const double *__restrict__ buf, double *out) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= gm) return;
    double s = 0.0;
    for (int p = 0; p < n_phase; ++p) s += buf[(long long)p * gm + k];
    out[k] = s;
}

// float -> double copy without FP64 instructions
__global__ void k_f32_widen(long long count, const float *__restrict__ a, double *__restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) out[i] = soap_f32_to_f64(a[i]);
}

namespace soapgb {

// Integration on device buffers (all pointers device).  temp/bi: n_phase x gm.
// out_stride: distance between phases in flux/bconv/tot (>= n).
// Outputs are float for the FP32 form (out_f32 must be set), double otherwise.
int integrate_device(soapgb_ctx *ctx, int form, int n, int n_eff, const double *d_wave, int grid, int n_phase,
                     const double *d_temp, const double *d_bi, const soapgb_maps &dm, const soapgb_cubes &dc,
                     double step, const soapgb_activity *act, void *d_flux, void *d_bconv, void *d_tot, int out_f32,
                     long long out_stride, int *d_cells, int *d_counts, char *fir_scratch,
                     const FirPlanSizes &fp) {
    if ((form == SOAPGB_FAST32) != (out_f32 != 0))
        return set_error(ctx, SOAPGB_ERR_ARG, "integration: FP32 outputs go with the FP32 form only");
    long long gm = (long long)grid * grid;
    if (form == SOAPGB_PLAIN64) {
        int rc = compact_cells(ctx, n_phase, (int)gm, d_bi, -0.5, 1.5, (int)gm, d_cells, d_counts);
        if (rc) return rc;
        dim3 g(grid_for(ctx, n, 256), n_phase);
        SOAP_TRACED(ctx, "integrate_plain64", k_phase_plain64<<<g, 256, 0, ctx->stream>>>(
            n, n_eff, d_wave, dc.q_norm, dc.q_sed, dc.spot_norm, dc.fac_norm, dc.spot_sed, dc.fac_sed, (int)gm,
            d_cells, d_counts, d_temp, d_bi, dm.delta, dm.limb, dm.lb, dm.region, gm, step, act->solar,
            act->t_star, act->t_diff_fac, (double *)d_flux, (double *)d_bconv, (double *)d_tot, out_stride, dc.n_mu,
            ctx->d_status));
        SOAP_LAUNCHED(ctx);
        return SOAPGB_OK;
    }
    FirPhaseArgs a;
    a.n = n;
    a.n_eff = n_eff;
    a.wave = d_wave;
    a.cubes = &dc;
    a.n_phase = n_phase;
    a.temp = d_temp;
    a.bi = d_bi;
    a.delta = dm.delta;
    a.limb = dm.limb;
    a.lb = dm.lb;
    a.region = dm.region;
    a.gm = gm;
    a.step = step;
    a.act = act;
    a.flux = d_flux;
    a.bconv = d_bconv;
    a.tot = d_tot;
    a.out_f32 = out_f32;
    a.out_stride = out_stride;
    return fir_phase(ctx, form, a, fir_scratch, fp);
}

}  // namespace soapgb

extern "C" int soapgb_phase_integrate(soapgb_ctx *ctx, int form, int n, int n_eff, const double *wave, int grid,
                                      int n_phase, const double *temp, const double *bi, const soapgb_maps *maps,
                                      const soapgb_cubes *cubes, double step, const soapgb_activity *act, int mem,
                                      double *flux, double *bconv, double *tot) {
    if (!ctx || !maps || !cubes || !act) return SOAPGB_ERR_ARG;
    if (n < 2 || n_eff < 2 || n_eff > n || grid < 1 || n_phase < 0 || cubes->n_mu < 1 || !(step > 0) || !wave ||
        !temp || !bi || !flux || !bconv || !tot || !maps->delta || !maps->limb || !maps->lb || !maps->region ||
        !cubes->q_norm || !cubes->q_sed || !cubes->spot_norm || !cubes->fac_norm || !cubes->spot_sed ||
        !cubes->fac_sed)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_phase_integrate: bad arguments");
    if (form != SOAPGB_PLAIN64 && form != SOAPGB_FAST64 && form != SOAPGB_FAST32)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_phase_integrate: unknown form %d", form);
    if (n_phase == 0) return SOAPGB_OK;
    SOAP_DEVICE(ctx);
    long long gm = (long long)grid * grid;
    int n_mu = cubes->n_mu;
    size_t cube_b = sizeof(double) * (size_t)n * n_mu;
    bool host = (mem == SOAPGB_HOST);
    Workspace ws(ctx);
    int s_wave = ws.add(host ? sizeof(double) * n : 0);
    int s_c[6];
    for (int q = 0; q < 4; ++q) s_c[q] = ws.add(host ? cube_b : 0);
    for (int q = 4; q < 6; ++q) s_c[q] = ws.add(host ? sizeof(double) * n : 0);
    int s_temp = ws.add(host ? sizeof(double) * gm * n_phase : 0);
    int s_bi = ws.add(host ? sizeof(double) * gm * n_phase : 0);
    int s_m[4];
    for (int q = 0; q < 3; ++q) s_m[q] = ws.add(host ? sizeof(double) * gm : 0);
    s_m[3] = ws.add(host ? sizeof(int) * gm : 0);
    int s_out[3];
    for (int q = 0; q < 3; ++q) s_out[q] = ws.add(host ? sizeof(double) * (size_t)n * n_phase : 0);
    int s_cells = ws.add(sizeof(int) * gm * n_phase);
    int s_counts = ws.add(sizeof(int) * n_phase);
    int s_f32 = ws.add(form == SOAPGB_FAST32 ? sizeof(float) * 3 * (size_t)n * n_phase : 0);
    FirPlanSizes fp = fir_plan_sizes(form, n, n_mu, gm, true, n_phase);
    int s_fir = ws.add(fp.bytes);
    int rc = ws.commit();
    if (rc) return rc;
#define STAGE(dst, src, bytes, slot)                                                           \
    dst = (decltype(dst))stage_in(ctx, mem, src, bytes, ws.get<void>(slot), &rc);             \
    if (rc) return rc;
    const double *d_wave;
    STAGE(d_wave, wave, sizeof(double) * n, s_wave);
    soapgb_cubes dc;
    dc.n_mu = n_mu;
    STAGE(dc.q_norm, cubes->q_norm, cube_b, s_c[0]);
    STAGE(dc.q_sed, cubes->q_sed, cube_b, s_c[1]);
    STAGE(dc.spot_norm, cubes->spot_norm, cube_b, s_c[2]);
    STAGE(dc.fac_norm, cubes->fac_norm, cube_b, s_c[3]);
    STAGE(dc.spot_sed, cubes->spot_sed, sizeof(double) * n, s_c[4]);
    STAGE(dc.fac_sed, cubes->fac_sed, sizeof(double) * n, s_c[5]);
    const double *d_temp, *d_bi;
    STAGE(d_temp, temp, sizeof(double) * gm * n_phase, s_temp);
    STAGE(d_bi, bi, sizeof(double) * gm * n_phase, s_bi);
    soapgb_maps dm;
    const double *cd;
    STAGE(cd, maps->delta, sizeof(double) * gm, s_m[0]);
    dm.delta = (double *)cd;
    STAGE(cd, maps->limb, sizeof(double) * gm, s_m[1]);
    dm.limb = (double *)cd;
    STAGE(cd, maps->lb, sizeof(double) * gm, s_m[2]);
    dm.lb = (double *)cd;
    const int *ci;
    STAGE(ci, maps->region, sizeof(int) * gm, s_m[3]);
    dm.region = (int *)ci;
    dm.mu = nullptr;
#undef STAGE
    double *d_flux = host ? ws.get<double>(s_out[0]) : flux;
    double *d_bconv = host ? ws.get<double>(s_out[1]) : bconv;
    double *d_tot = host ? ws.get<double>(s_out[2]) : tot;
    if (form == SOAPGB_FAST32) {
        float *f32 = ws.get<float>(s_f32);
        size_t pn = (size_t)n * n_phase;
        rc = integrate_device(ctx, form, n, n_eff, d_wave, grid, n_phase, d_temp, d_bi, dm, dc, step, act, f32,
                              f32 + pn, f32 + 2 * pn, 1, n, ws.get<int>(s_cells), ws.get<int>(s_counts),
                              ws.get<char>(s_fir), fp);
        if (rc) return rc;
        double *outs[3] = {d_flux, d_bconv, d_tot};
        for (int q = 0; q < 3; ++q) {
            SOAP_TRACED(ctx, "widen", k_f32_widen<<<grid_for(ctx, (long long)pn, 256), 256, 0, ctx->stream>>>((long long)pn, f32 + q * pn, outs[q]));
            SOAP_LAUNCHED(ctx);
        }
    } else {
        rc = integrate_device(ctx, form, n, n_eff, d_wave, grid, n_phase, d_temp, d_bi, dm, dc, step, act, d_flux,
                              d_bconv, d_tot, 0, n, ws.get<int>(s_cells), ws.get<int>(s_counts), ws.get<char>(s_fir),
                              fp);
        if (rc) return rc;
    }
    if (host) {
        size_t ob = sizeof(double) * (size_t)n * n_phase;
        SOAP_CUDA(ctx, cudaMemcpyAsync(flux, d_flux, ob, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(bconv, d_bconv, ob, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(tot, d_tot, ob, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return host ? check_status(ctx, "soapgb_phase_integrate") : SOAPGB_OK;
}

extern "C" int soapgb_phase_integrate_adjoint(soapgb_ctx *ctx, int n, int n_eff, const double *wave, int grid,
                                              int n_phase, const double *temp, const double *bi,
                                              const soapgb_maps *maps, const soapgb_cubes *cubes, double step,
                                              const soapgb_activity *act, const double *g_flux,
                                              const double *g_bconv, const double *g_tot, int mem,
                                              double *grad_q_norm, double *grad_q_sed, double *grad_spot_norm,
                                              double *grad_fac_norm, double *grad_spot_sed, double *grad_fac_sed,
                                              double *grad_limb, double *grad_delta) {
    if (!ctx || !maps || !cubes || !act) return SOAPGB_ERR_ARG;
    if (n < 2 || n_eff < 2 || n_eff > n || grid < 1 || n_phase < 0 || cubes->n_mu < 1 ||
        cubes->n_mu > ADJ_MAX_MU || !(step > 0) || !wave || !temp || !bi || !maps->delta || !maps->limb ||
        !maps->lb || !maps->region || !cubes->q_norm || !cubes->q_sed || !cubes->spot_norm || !cubes->fac_norm ||
        !cubes->spot_sed || !cubes->fac_sed || (!g_flux != !g_tot) || !g_bconv || !grad_q_norm || !grad_q_sed ||
        !grad_spot_norm || !grad_fac_norm || !grad_spot_sed || !grad_fac_sed || !grad_limb || !grad_delta)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_phase_integrate_adjoint: bad arguments");
    SOAP_DEVICE(ctx);
    const long long gm = (long long)grid * grid;
    const int n_mu = cubes->n_mu;
    const size_t cube_b = sizeof(double) * (size_t)n * n_mu, row_b = sizeof(double) * (size_t)n;
    const size_t g_b = sizeof(double) * (size_t)n * std::max(n_phase, 1);
    const size_t map_b = sizeof(double) * (size_t)gm * std::max(n_phase, 1);
    const bool host = (mem == SOAPGB_HOST);
    Workspace ws(ctx);
    int s_wave = ws.add(host ? row_b : 0);
    int s_c[6];
    for (int q = 0; q < 4; ++q) s_c[q] = ws.add(host ? cube_b : 0);
    for (int q = 4; q < 6; ++q) s_c[q] = ws.add(host ? row_b : 0);
    int s_temp = ws.add(host ? map_b : 0), s_bi = ws.add(host ? map_b : 0);
    int s_m[4];
    for (int q = 0; q < 3; ++q) s_m[q] = ws.add(host ? sizeof(double) * gm : 0);
    s_m[3] = ws.add(host ? sizeof(int) * gm : 0);
    int s_g[3];
    for (int q = 0; q < 3; ++q) s_g[q] = ws.add(host ? g_b : 0);
    int s_o[8];
    for (int q = 0; q < 4; ++q) s_o[q] = ws.add(host ? cube_b : 0);
    for (int q = 4; q < 6; ++q) s_o[q] = ws.add(host ? row_b : 0);
    s_o[6] = ws.add(host ? sizeof(double) * gm : 0);
    s_o[7] = ws.add(host ? sizeof(double) * gm : 0);
    int s_cells = ws.add(sizeof(int) * gm * std::max(n_phase, 1));
    int s_rcells = ws.add(sizeof(int) * gm * std::max(n_phase, 1));
    int s_counts = ws.add(sizeof(int) * std::max(n_phase, 1));
    int s_roff = ws.add(sizeof(int) * (size_t)(n_mu + 1) * std::max(n_phase, 1));
    int s_buf = ws.add(map_b), s_bufd = ws.add(map_b);
    // no flux or tot gradients: one zero array stands in for both, and the continuum
    // rows, which enter only flux and tot, get no pass
    const bool bconv_only = (g_flux == nullptr);
    int s_zero = ws.add(bconv_only ? g_b : 0);
    int s_inv = ws.add(row_b);
    int rc = ws.commit();
    if (rc) return rc;
#define STAGE(dst, src, bytes, slot)                                                           \
    dst = (decltype(dst))stage_in(ctx, mem, src, bytes, ws.get<void>(slot), &rc);             \
    if (rc) return rc;
    const double *d_wave, *d_qn, *d_qs, *d_sn, *d_fn, *d_ss, *d_fs, *d_temp, *d_bi, *d_delta, *d_limb, *d_lb;
    const int *d_region;
    const double *d_gf, *d_gb, *d_gt;
    STAGE(d_wave, wave, row_b, s_wave);
    STAGE(d_qn, cubes->q_norm, cube_b, s_c[0]);
    STAGE(d_qs, cubes->q_sed, cube_b, s_c[1]);
    STAGE(d_sn, cubes->spot_norm, cube_b, s_c[2]);
    STAGE(d_fn, cubes->fac_norm, cube_b, s_c[3]);
    STAGE(d_ss, cubes->spot_sed, row_b, s_c[4]);
    STAGE(d_fs, cubes->fac_sed, row_b, s_c[5]);
    STAGE(d_temp, temp, map_b, s_temp);
    STAGE(d_bi, bi, map_b, s_bi);
    STAGE(d_delta, maps->delta, sizeof(double) * gm, s_m[0]);
    STAGE(d_limb, maps->limb, sizeof(double) * gm, s_m[1]);
    STAGE(d_lb, maps->lb, sizeof(double) * gm, s_m[2]);
    STAGE(d_region, maps->region, sizeof(int) * gm, s_m[3]);
    STAGE(d_gf, g_flux, g_b, s_g[0]);
    STAGE(d_gb, g_bconv, g_b, s_g[1]);
    STAGE(d_gt, g_tot, g_b, s_g[2]);
#undef STAGE
    if (bconv_only) {
        SOAP_CUDA(ctx, cudaMemsetAsync(ws.get<void>(s_zero), 0, g_b, ctx->stream));
        d_gf = d_gt = ws.get<double>(s_zero);
    }
    double *o_qn = host ? ws.get<double>(s_o[0]) : grad_q_norm;
    double *o_qs = host ? ws.get<double>(s_o[1]) : grad_q_sed;
    double *o_sn = host ? ws.get<double>(s_o[2]) : grad_spot_norm;
    double *o_fn = host ? ws.get<double>(s_o[3]) : grad_fac_norm;
    double *o_ss = host ? ws.get<double>(s_o[4]) : grad_spot_sed;
    double *o_fs = host ? ws.get<double>(s_o[5]) : grad_fac_sed;
    double *o_lm = host ? ws.get<double>(s_o[6]) : grad_limb;
    double *o_dl = host ? ws.get<double>(s_o[7]) : grad_delta;
    int *d_cells = ws.get<int>(s_cells), *d_rcells = ws.get<int>(s_rcells);
    int *d_counts = ws.get<int>(s_counts), *d_roff = ws.get<int>(s_roff);
    double *d_buf = ws.get<double>(s_buf), *d_bufd = ws.get<double>(s_bufd);
    double *d_inv = ws.get<double>(s_inv);
    if (n_phase == 0) {
        for (double *o : {o_qn, o_qs, o_sn, o_fn})
            SOAP_CUDA(ctx, cudaMemsetAsync(o, 0, cube_b, ctx->stream));
        SOAP_CUDA(ctx, cudaMemsetAsync(o_ss, 0, row_b, ctx->stream));
        SOAP_CUDA(ctx, cudaMemsetAsync(o_fs, 0, row_b, ctx->stream));
        SOAP_CUDA(ctx, cudaMemsetAsync(o_lm, 0, sizeof(double) * gm, ctx->stream));
        SOAP_CUDA(ctx, cudaMemsetAsync(o_dl, 0, sizeof(double) * gm, ctx->stream));
    } else {
        rc = compact_cells(ctx, n_phase, (int)gm, d_bi, -0.5, 1.5, (int)gm, d_cells, d_counts);
        if (rc) return rc;
        k_adj_bucket<<<n_phase, 32, 0, ctx->stream>>>(n_mu, gm, d_cells, d_counts, d_region, d_rcells, d_roff,
                                                      ctx->d_status);
        SOAP_LAUNCHED(ctx);
        k_adj_inv<<<grid_for(ctx, n_eff, 256), 256, 0, ctx->stream>>>(n_eff, d_wave, d_inv);
        SOAP_LAUNCHED(ctx);
        SOAP_TRACED(ctx, "adjoint_rows",
                    (bconv_only ? k_adj_rows<true> : k_adj_rows<false>)<<<dim3(grid_for(ctx, n, 256), n_mu), 256, 0,
                                                                              ctx->stream>>>(
                        n, n_eff, d_wave, d_inv, d_ss, d_fs, n_phase, gm, d_rcells, d_roff, n_mu, d_temp, d_bi, d_delta,
                        d_limb, d_lb, step, act->solar, act->t_star, act->t_diff_fac, d_gf, d_gb, d_gt, n, o_qn, o_qs,
                        o_sn, o_fn));
        SOAP_LAUNCHED(ctx);
        if (bconv_only) {
            SOAP_CUDA(ctx, cudaMemsetAsync(o_ss, 0, row_b, ctx->stream));
            SOAP_CUDA(ctx, cudaMemsetAsync(o_fs, 0, row_b, ctx->stream));
        } else {
            SOAP_TRACED(ctx, "adjoint_continuum",
                        k_adj_continuum<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(
                            n, n_eff, d_wave, d_inv, d_qn, d_sn, d_fn, d_ss, d_fs, n_phase, gm, d_cells, d_counts, d_temp,
                            d_bi, d_delta, d_limb, d_lb, d_region, n_mu, step, act->solar, act->t_star,
                            act->t_diff_fac, d_gf, d_gt, n, o_ss, o_fs));
            SOAP_LAUNCHED(ctx);
        }
        SOAP_CUDA(ctx, cudaMemsetAsync(d_buf, 0, map_b, ctx->stream));
        SOAP_CUDA(ctx, cudaMemsetAsync(d_bufd, 0, map_b, ctx->stream));
        const int gx = (int)std::min<long long>(gm, 4LL * std::max(ctx->num_sms, 1));
        SOAP_TRACED(ctx, "adjoint_limb",
                    (bconv_only ? k_adj_limb<true> : k_adj_limb<false>)<<<dim3(gx, n_phase), 256, 0, ctx->stream>>>(
                        n, n_eff, d_wave, d_inv, d_qn, d_qs, d_sn, d_fn, d_ss, d_fs, gm, d_cells, d_counts, d_temp, d_bi,
                        d_delta, d_lb, d_region, n_mu, step, act->solar, act->t_star, act->t_diff_fac, d_gf, d_gb,
                        d_gt, n, d_limb, d_buf, d_bufd));
        SOAP_LAUNCHED(ctx);
        k_adj_sum_phases<<<grid_for(ctx, gm, 256), 256, 0, ctx->stream>>>(n_phase, gm, d_buf, o_lm);
        SOAP_LAUNCHED(ctx);
        k_adj_sum_phases<<<grid_for(ctx, gm, 256), 256, 0, ctx->stream>>>(n_phase, gm, d_bufd, o_dl);
        SOAP_LAUNCHED(ctx);
    }
    if (host) {
        SOAP_CUDA(ctx, cudaMemcpyAsync(grad_q_norm, o_qn, cube_b, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(grad_q_sed, o_qs, cube_b, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(grad_spot_norm, o_sn, cube_b, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(grad_fac_norm, o_fn, cube_b, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(grad_spot_sed, o_ss, row_b, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(grad_fac_sed, o_fs, row_b, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(grad_limb, o_lm, sizeof(double) * gm, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaMemcpyAsync(grad_delta, o_dl, sizeof(double) * gm, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return check_status(ctx, "soapgb_phase_integrate_adjoint");
    }
    return SOAPGB_OK;
}
