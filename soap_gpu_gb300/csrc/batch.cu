// Batched form: many stars of uneven sizes through the per-phase path in one job.
//
// Reference: run_all_SOAP.py runs one star per invocation -- SOAP_initialize twice, then
// SOAP_integration and SOAP_resolution over the star's phases (run_all_SOAP.py:226-250,
// the phase loop of SOAP_integration.cu:661-845).  Here a batch of stars shares the seed
// spectra and the wavelength grid; per star the disk maps, the two quiet spectra, the
// phase lists and the tile plans are built, then the active-region integration of every
// visible phase of every star runs in ONE persistent launch over (star, phase, tile)
// items, and each star's spectra are convolved and normalised against its own quiet
// spectra.
//
// soapgb_batch_create does all the host-side work (region tables, visibility, sizes,
// uploads) and owns the batch's device memory; soapgb_batch_run only enqueues kernels and
// device-to-device copies on the context's stream, reads no host memory and synchronises
// nothing, so it can be captured in a CUDA graph and replayed.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "internal.cuh"
#include "fir.cuh"
#include "regions.cuh"
#include "resolution.cuh"

using namespace soapgb;

namespace soapgb {
void disk_omega_host(const soapgb_star *st, std::vector<double> &ov, double &sin_incl);
int disk_maps_launch(soapgb_ctx *ctx, const soapgb_star *star, int n_mu, const double *d_mu, const double *d_ov,
                     double sin_incl, double *delta, double *limb, double *mu, int *region, double *lb);
}  // namespace soapgb

namespace {

struct BatchStar {
    soapgb_star star;
    int n_phase = 0, n_run = 0, box_cap = 0;
    long long gm = 0;
    long long phase0 = 0;            // first row of the star's phases in the batch output
    double sin_incl = 0.0;
    // device
    double *ov = nullptr;            // per-row rotation constants
    double *delta = nullptr, *limb = nullptr, *mu = nullptr, *lb = nullptr;
    int *region = nullptr;
    double *q_sed = nullptr, *q_norm = nullptr;   // quiet spectra, n each
    char *fir = nullptr;             // geometry / lists / plans (typed cubes shared)
    float *raw = nullptr;            // FP32 deficits [phase][tot, flux, bconv][n]
    char *small = nullptr;           // region table, run / zero lists, zero flags, convolution rows
    const RegionPhase *table = nullptr;
    const int *roff = nullptr;
    int *lists = nullptr;            // run list then zero list
    unsigned char *zspec = nullptr;  // [3 n_phase]: 1 for the spectra of phases without a visible region
    int *blist = nullptr;            // the non-zero spectra (the convolution's rows)
    int n_blist = 0;
    // host
    std::vector<int> h_lists;
    std::vector<unsigned char> h_zspec;
    soapgb_maps maps;
    FirPhaseArgs fa;
    FirPlanSizes fp;
};

size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

struct soapgb_batch {
    int device = 0;
    int form = SOAPGB_FAST32;
    int n = 0, n_eff = 0, n_mu = 0;
    double step = 0, sigma_v = 0, conv_step = 0, sentinel = 0;
    double w3[3] = {0, 0, 0};
    soapgb_activity act{};
    const double *wave = nullptr;    // caller's device arrays
    soapgb_cubes cubes{};
    std::vector<BatchStar> stars;
    long long total_phases = 0;
    // device memory owned by the batch
    char *mem = nullptr;
    size_t bytes = 0;
    double *mu_b = nullptr;
    char *typed_mem = nullptr;
    FirTyped typed{};
    // worker streams: the per-star stages of star s run on worker s % n_work, so that the
    // small launches of different stars overlap; each worker has its own quiet-disk and
    // convolution workspaces, used by its stars in turn
    int n_work = 1;
    std::vector<cudaStream_t> work;
    std::vector<cudaEvent_t> fork_ev, join_ev;   // [2]: before / after the integration; [2 n_work]
    std::vector<char *> quiet_ws;
    FirPlanSizes quiet_fp;
    std::vector<char *> res_ws;
    char *star_args = nullptr;       // the integration kernel's per-star arguments
    int2 *items = nullptr;           // (star, phase) of every visible phase
    int n_items = 0;
    std::vector<char> star0_args;
    int chunk = 0, blocks_per_sm = 0;
};

namespace {

int batch_error(soapgb_ctx *ctx, const char *what) { return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_batch_create: %s", what); }

// carve `bytes` from the batch memory at *off (256-byte aligned)
char *take(soapgb_batch *b, size_t &off, size_t bytes) {
    char *p = b->mem + off;
    off += al256(bytes);
    return p;
}

}  // namespace

extern "C" int soapgb_batch_create(soapgb_ctx *ctx, const soapgb_batch_desc *d, soapgb_batch **out) {
    if (!ctx || !d || !out) return SOAPGB_ERR_ARG;
    *out = nullptr;
    if (d->n < 3 || d->n_eff < 2 || d->n_eff > d->n || !d->wave || !d->cubes || d->n_star < 1 || !d->stars ||
        !d->phase_offsets || !d->phases || !d->reg_offsets || !(d->step > 0) || !(d->sigma_v > 0) ||
        !(d->conv_step > 0) || d->cubes->n_mu < 1 || (d->cubes->n_mu > 1 && !d->mu_boundary))
        return batch_error(ctx, "bad arguments");
    if (d->form != SOAPGB_FAST32) return batch_error(ctx, "the batched form runs the FP32 form only");
    SOAP_DEVICE(ctx);
    std::unique_ptr<soapgb_batch> b(new soapgb_batch());
    b->device = ctx->device;
    b->form = d->form;
    b->n = d->n;
    b->n_eff = d->n_eff;
    b->n_mu = d->cubes->n_mu;
    b->step = d->step;
    b->sigma_v = d->sigma_v;
    b->conv_step = d->conv_step;
    b->sentinel = d->sentinel;
    b->act = d->act;
    b->wave = d->wave;
    b->cubes = *d->cubes;
    b->chunk = d->chunk;
    b->blocks_per_sm = d->blocks_per_sm;
    // the wavelength edges: read once here, so that the run reads no host memory
    SOAP_CUDA(ctx, cudaMemcpyAsync(b->w3, d->wave, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SOAP_CUDA(ctx, cudaMemcpyAsync(b->w3 + 2, d->wave + d->n_eff - 1, sizeof(double), cudaMemcpyDeviceToHost,
                                   ctx->stream));
    SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const int n = b->n, n_eff = b->n_eff, n_mu = b->n_mu;
    if (d->phase_offsets[0] != 0) return batch_error(ctx, "phase_offsets[0] must be 0");
    b->stars.resize(d->n_star);
    long long max_gm = 0, max_spec = 0;
    // region tables, visibility and sizes of every star (host)
    std::vector<std::vector<char>> packs(d->n_star);
    std::vector<size_t> off_lists(d->n_star), off_zspec(d->n_star), off_blist(d->n_star), pm_bytes(d->n_star);
    std::vector<size_t> off_roff(d->n_star, 0);   // the region offsets' place in the table image
    for (int s = 0; s < d->n_star; ++s) {
        BatchStar &st = b->stars[s];
        st.star = d->stars[s];
        const int p0 = d->phase_offsets[s], p1 = d->phase_offsets[s + 1];
        if (p1 < p0) return batch_error(ctx, "phase_offsets must not decrease");
        st.n_phase = p1 - p0;
        st.phase0 = p0;
        const int G = st.star.grid;
        if (G < 4 || G > 20000) return batch_error(ctx, "a star's grid is out of range");
        st.gm = (long long)G * G;
        if (st.gm > fir_box_lists_max_gm()) return batch_error(ctx, "a star's grid is above the box-list limit");
        max_gm = std::max(max_gm, st.gm);
        max_spec = std::max(max_spec, 3LL * st.n_phase);
        if (st.n_phase == 0) continue;
        const int *roff = d->reg_offsets + p0;
        std::vector<int> h_off(st.n_phase + 1);
        for (int q = 0; q <= st.n_phase; ++q) h_off[q] = roff[q] - roff[0];
        const int n_rows = h_off[st.n_phase];
        if (n_rows < 0) return batch_error(ctx, "reg_offsets must not decrease");
        if (n_rows > 0 && !d->regions) return batch_error(ctx, "null regions");
        pm_bytes[s] = phase_maps_scratch_bytes(n_rows, st.n_phase);
        std::vector<unsigned char> vis;
        long long max_box = 0;
        const RegionPhase *dt = nullptr;
        const int *dr = nullptr;
        int rc = phase_table_device(ctx, G, st.star.incl, st.n_phase, d->phases + p0, h_off.data(),
                                    d->regions + 4 * (size_t)roff[0], &b->act, nullptr, pm_bytes[s], &dt, &dr, &vis,
                                    &max_box, &packs[s]);
        if (rc) return rc;
        // with an image requested, the table's addresses are offsets from a null base
        off_roff[s] = (size_t)(reinterpret_cast<uintptr_t>(dr) - reinterpret_cast<uintptr_t>(dt));
        for (int p = 0; p < st.n_phase; ++p)
            if (vis[p]) st.h_lists.push_back(p);
        st.n_run = (int)st.h_lists.size();
        for (int p = 0; p < st.n_phase; ++p)
            if (!vis[p]) st.h_lists.push_back(p);
        st.h_zspec.assign(3 * (size_t)st.n_phase, 0);
        for (int p = 0; p < st.n_phase; ++p)
            st.h_zspec[3 * p] = st.h_zspec[3 * p + 1] = st.h_zspec[3 * p + 2] = vis[p] ? 0 : 1;
        st.box_cap = fir_sorted_box_capacity(max_box);
        off_lists[s] = al256(pm_bytes[s]);
        off_zspec[s] = off_lists[s] + al256(sizeof(int) * st.n_phase);
        off_blist[s] = off_zspec[s] + al256(3 * (size_t)st.n_phase);
        st.fp = fir_plan_sizes(b->form, n, n_mu, st.gm, true, st.n_phase, true);
    }
    b->total_phases = d->phase_offsets[d->n_star];
    // sizes
    b->n_work = std::max(1, std::min(4, d->n_star));
    b->quiet_fp = fir_plan_sizes(b->form, n, n_mu, max_gm, false, 1);
    const size_t res_b = resolution_scratch_bytes(b->form, n, n_eff, (int)std::max(3LL, max_spec));
    size_t total = al256(sizeof(double) * (n_mu > 1 ? n_mu - 1 : 1)) + al256(fir_typed_bytes(b->form, n, n_mu)) +
                   b->n_work * (al256(b->quiet_fp.bytes) + al256(res_b)) +
                   al256(fir_tile_args_bytes() * d->n_star) + al256(sizeof(int2) * (size_t)std::max(1LL, b->total_phases));
    for (auto &st : b->stars) {
        total += al256(sizeof(double) * st.star.grid) + 4 * al256(sizeof(double) * st.gm) + al256(sizeof(int) * st.gm) +
                 2 * al256(sizeof(double) * n);
        if (st.n_phase == 0) continue;
        total += al256(st.fp.bytes) + al256(sizeof(float) * 3 * (size_t)n * st.n_phase);
        total += al256(off_blist[&st - &b->stars[0]] + sizeof(int) * (3 * (size_t)st.n_phase + 2));
    }
    cudaError_t e = cudaMalloc((void **)&b->mem, total);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(ctx, SOAPGB_ERR_ALLOC, "soapgb_batch_create: %zu bytes of device memory not available", total);
    }
    b->bytes = total;
    size_t off = 0;
    b->mu_b = (double *)take(b.get(), off, sizeof(double) * (n_mu > 1 ? n_mu - 1 : 1));
    if (n_mu > 1)
        SOAP_CUDA(ctx, cudaMemcpyAsync(b->mu_b, d->mu_boundary, sizeof(double) * (n_mu - 1), cudaMemcpyHostToDevice,
                                       ctx->stream));
    b->typed_mem = take(b.get(), off, fir_typed_bytes(b->form, n, n_mu));
    for (int w = 0; w < b->n_work; ++w) {
        b->quiet_ws.push_back(take(b.get(), off, b->quiet_fp.bytes));
        b->res_ws.push_back(take(b.get(), off, res_b));
    }
    b->star_args = take(b.get(), off, fir_tile_args_bytes() * d->n_star);
    b->items = (int2 *)take(b.get(), off, sizeof(int2) * (size_t)std::max(1LL, b->total_phases));
    // the typed cubes' addresses are fixed by the layout (they are written by the run)
    fir_typed_layout(b->form, n, n_mu, b->typed_mem, b->cubes, &b->typed);
    std::vector<char> args(fir_tile_args_bytes() * d->n_star, 0);
    std::vector<int2> items;
    std::vector<std::vector<double>> ovs(d->n_star);
    for (int s = 0; s < d->n_star; ++s) {
        BatchStar &st = b->stars[s];
        const int G = st.star.grid;
        st.ov = (double *)take(b.get(), off, sizeof(double) * G);
        disk_omega_host(&st.star, ovs[s], st.sin_incl);
        SOAP_CUDA(ctx, cudaMemcpyAsync(st.ov, ovs[s].data(), sizeof(double) * G, cudaMemcpyHostToDevice, ctx->stream));
        st.delta = (double *)take(b.get(), off, sizeof(double) * st.gm);
        st.limb = (double *)take(b.get(), off, sizeof(double) * st.gm);
        st.mu = (double *)take(b.get(), off, sizeof(double) * st.gm);
        st.lb = (double *)take(b.get(), off, sizeof(double) * st.gm);
        st.region = (int *)take(b.get(), off, sizeof(int) * st.gm);
        st.q_sed = (double *)take(b.get(), off, sizeof(double) * n);
        st.q_norm = (double *)take(b.get(), off, sizeof(double) * n);
        st.maps.delta = st.delta;
        st.maps.limb = st.limb;
        st.maps.mu = st.mu;
        st.maps.lb = st.lb;
        st.maps.region = st.region;
        if (st.n_phase == 0) continue;
        st.fir = take(b.get(), off, st.fp.bytes);
        st.raw = (float *)take(b.get(), off, sizeof(float) * 3 * (size_t)n * st.n_phase);
        // the small uploads: region table, lists, zero flags, the convolution's rows
        std::vector<char> &pack = packs[s];
        std::vector<int> bl;
        for (long long q = 0; q < 3LL * st.n_phase; ++q)
            if (!st.h_zspec[q]) bl.push_back((int)q);
        st.n_blist = (int)bl.size();
        const size_t used = off_blist[s] + sizeof(int) * bl.size();
        st.small = take(b.get(), off, off_blist[s] + sizeof(int) * (3 * (size_t)st.n_phase + 2));
        pack.resize(std::max(pack.size(), used), 0);
        memcpy(pack.data() + off_lists[s], st.h_lists.data(), sizeof(int) * st.n_phase);
        memcpy(pack.data() + off_zspec[s], st.h_zspec.data(), 3 * (size_t)st.n_phase);
        if (!bl.empty()) memcpy(pack.data() + off_blist[s], bl.data(), sizeof(int) * bl.size());
        SOAP_CUDA(ctx, cudaMemcpyAsync(st.small, pack.data(), used, cudaMemcpyHostToDevice, ctx->stream));
        st.table = (const RegionPhase *)st.small;   // the table rows, then the offsets
        st.roff = (const int *)(st.small + off_roff[s]);
        st.lists = (int *)(st.small + off_lists[s]);
        st.zspec = (unsigned char *)(st.small + off_zspec[s]);
        st.blist = (int *)(st.small + off_blist[s]);
        // the star's integration arguments (its geometry stage and the shared launch)
        FirPhaseArgs &fa = st.fa;
        fa.n = n;
        fa.n_eff = n_eff;
        fa.wave = b->wave;
        fa.cubes = &b->cubes;
        fa.n_phase = st.n_phase;
        fa.table = st.table;
        fa.reg_off = st.roff;
        fa.grid = G;
        fa.box_cap = st.box_cap;
        fa.run_list = st.lists;
        fa.zero_list = st.lists + st.n_run;
        fa.run_host = st.h_lists.data();
        fa.zero_host = st.h_lists.data() + st.n_run;
        fa.n_run = st.n_run;
        fa.n_zero = st.n_phase - st.n_run;
        fa.zero_fill = 0;
        fa.delta = st.delta;
        fa.limb = st.limb;
        fa.lb = st.lb;
        fa.region = st.region;
        fa.gm = st.gm;
        fa.step = b->step;
        fa.act = &b->act;
        fa.tot = st.raw;
        fa.flux = st.raw + n;
        fa.bconv = st.raw + 2 * (size_t)n;
        fa.out_f32 = 1;
        fa.out_stride = 3LL * n;
        fa.lambda0 = b->w3[0];
        fa.typed = &b->typed;
        int rc = fir_phase_star_args(ctx, b->form, fa, st.fir, args.data() + fir_tile_args_bytes() * s);
        if (rc) return rc;
        for (int r = 0; r < st.n_run; ++r) items.push_back(make_int2(s, st.h_lists[r]));
    }
    b->n_items = (int)items.size();
    SOAP_CUDA(ctx, cudaMemcpyAsync(b->star_args, args.data(), args.size(), cudaMemcpyHostToDevice, ctx->stream));
    if (!items.empty())
        SOAP_CUDA(ctx, cudaMemcpyAsync(b->items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice,
                                       ctx->stream));
    // the first star with phases gives the launch its grid-wide fields
    b->star0_args.assign(args.begin(), args.begin() + fir_tile_args_bytes());
    for (int s = 0; s < d->n_star; ++s)
        if (b->stars[s].n_phase > 0) {
            b->star0_args.assign(args.begin() + fir_tile_args_bytes() * s,
                                 args.begin() + fir_tile_args_bytes() * (s + 1));
            break;
        }
    // the uploads read host vectors that end with this call
    SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int w = 0; w < b->n_work; ++w) {
        cudaStream_t st = nullptr;
        SOAP_CUDA(ctx, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        b->work.push_back(st);
    }
    for (int q = 0; q < 2 + 2 * b->n_work; ++q) {
        cudaEvent_t e = nullptr;
        SOAP_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        (q < 2 ? b->fork_ev : b->join_ev).push_back(e);
    }
    *out = b.release();
    return SOAPGB_OK;
}

extern "C" int soapgb_batch_tune(soapgb_batch *b, int chunk, int blocks_per_sm) {
    if (!b || chunk < 0 || blocks_per_sm < 0) return SOAPGB_ERR_ARG;
    b->chunk = chunk;
    b->blocks_per_sm = blocks_per_sm;
    return SOAPGB_OK;
}

extern "C" size_t soapgb_batch_device_bytes(const soapgb_batch *b) { return b ? b->bytes : 0; }

extern "C" long long soapgb_batch_items(const soapgb_batch *b) { return b ? b->n_items : -1; }

extern "C" int soapgb_batch_run(soapgb_ctx *ctx, soapgb_batch *b, double *lower, double *quiet) {
    if (!ctx || !b || !lower) return SOAPGB_ERR_ARG;
    if (b->device != ctx->device) return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_batch_run: batch of another device");
    SOAP_DEVICE(ctx);
    const int n = b->n, n_eff = b->n_eff, n_mu = b->n_mu;
    int rc = SOAPGB_OK;
    // the shared typed cubes
    {
        FirTyped t;
        rc = fir_typed_cubes(ctx, b->form, n, b->cubes, b->typed_mem, &t);
        if (rc) return rc;
    }
    // fork the workers off the context's stream
    auto fork = [&](int f) -> int {
        SOAP_CUDA(ctx, cudaEventRecord(b->fork_ev[f], ctx->stream));
        for (auto w : b->work) SOAP_CUDA(ctx, cudaStreamWaitEvent(w, b->fork_ev[f], 0));
        return SOAPGB_OK;
    };
    auto join = [&](int f) -> int {
        for (int w = 0; w < b->n_work; ++w) {
            cudaEvent_t e = b->join_ev[f * b->n_work + w];
            SOAP_CUDA(ctx, cudaEventRecord(e, b->work[w]));
            SOAP_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, e, 0));
        }
        return SOAPGB_OK;
    };
    rc = fork(0);
    if (rc) return rc;
    // per star, on its worker: disk maps, both quiet spectra (one set of lists), geometry
    // (cell geometry, lists, prefix sums, tile plans)
    for (size_t s = 0; s < b->stars.size(); ++s) {
        BatchStar &st = b->stars[s];
        const int w = (int)(s % b->n_work);
        AuxScope on(ctx, b->work[w]);
        rc = disk_maps_launch(ctx, &st.star, n_mu, b->mu_b, st.ov, st.sin_incl, st.delta, st.limb, st.mu, st.region,
                              st.lb);
        if (rc) return rc;
        FirQuietArgs qa;
        qa.n = n;
        qa.n_eff = n_eff;
        qa.wave = b->wave;
        qa.cube = b->cubes.q_sed;
        qa.cube2 = b->cubes.q_norm;
        qa.n_mu = n_mu;
        qa.gm = st.gm;
        qa.delta = st.delta;
        qa.limb = st.limb;
        qa.region = st.region;
        qa.step = b->step;
        qa.out = st.q_sed;
        qa.out2 = st.q_norm;
        qa.lambda0 = b->w3[0];
        rc = fir_quiet(ctx, b->form, qa, b->quiet_ws[w], b->quiet_fp);
        if (rc) return rc;
        if (st.n_run == 0) continue;
        st.fa.stage = FIR_STAGE_GEOMETRY;
        rc = fir_phase(ctx, b->form, st.fa, st.fir, st.fp);
        if (rc) return rc;
    }
    rc = join(0);
    if (rc) return rc;
    // the integration of every visible phase of every star: one launch
    rc = fir_phase_multi(ctx, b->form, b->star0_args.data(), b->star_args, b->items, b->n_items, b->chunk,
                         b->blocks_per_sm);
    if (rc) return rc;
    rc = fork(1);
    if (rc) return rc;
    // per star, on its worker: convolution and normalisation against its own quiet spectra
    for (size_t s = 0; s < b->stars.size(); ++s) {
        BatchStar &st = b->stars[s];
        if (st.n_phase == 0) continue;
        const int w = (int)(s % b->n_work);
        AuxScope on(ctx, b->work[w]);
        const int n_spec = 3 * st.n_phase;
        Res32 R;
        rc = resolution32_prepare(ctx, n, n_eff, n_spec, b->wave, b->w3[0], b->w3[1], b->w3[2], st.q_sed, st.q_norm, 3,
                                  b->sigma_v, 50.0, b->conv_step, b->conv_step, b->sentinel, b->res_ws[w], R);
        if (rc) return rc;
        rc = resolution32_run(ctx, R, st.raw, n, 0, n_spec, lower + (size_t)3 * st.phase0 * n_eff, n_eff, nullptr,
                              st.zspec, st.h_zspec.data(), ZeroRows::NORM, st.blist, st.n_blist);
        if (rc) return rc;
    }
    rc = join(1);
    if (rc) return rc;
    if (quiet) {
        for (size_t s = 0; s < b->stars.size(); ++s) {
            SOAP_CUDA(ctx, cudaMemcpyAsync(quiet + 2 * s * n, b->stars[s].q_sed, sizeof(double) * n,
                                           cudaMemcpyDeviceToDevice, ctx->stream));
            SOAP_CUDA(ctx, cudaMemcpyAsync(quiet + (2 * s + 1) * n, b->stars[s].q_norm, sizeof(double) * n,
                                           cudaMemcpyDeviceToDevice, ctx->stream));
        }
    }
    return SOAPGB_OK;
}

extern "C" int soapgb_batch_destroy(soapgb_batch *b) {
    if (!b) return SOAPGB_OK;
    {
        DeviceGuard g(b->device);
        for (auto w : b->work) cudaStreamSynchronize(w);
        for (auto w : b->work) cudaStreamDestroy(w);
        for (auto e : b->fork_ev) cudaEventDestroy(e);
        for (auto e : b->join_ev) cudaEventDestroy(e);
        if (b->mem) {
            cudaDeviceSynchronize();
            cudaFree(b->mem);
        }
    }
    delete b;
    return SOAPGB_OK;
}
