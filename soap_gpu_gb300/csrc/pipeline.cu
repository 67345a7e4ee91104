// Composite per-phase pipeline: maps -> integration -> convolution/normalisation.
//
// Reference: the SOAP_integration and SOAP_resolution processes spawned by
// run_all_SOAP.py:237-250, which hand the raw deficit spectra over through one
// float64 file per phase and type (SOAP_integration.cu:802-817 ->
// SOAP_resolution.cu:398-412).  Here the deficits stay in device memory and all
// phases go through each stage in one launch.
#include <algorithm>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "internal.cuh"
#include "fir.cuh"
#include "regions.cuh"
#include "resolution.cuh"

using namespace soapgb;

namespace soapgb {
int phase_maps_device(soapgb_ctx *ctx, int grid, double incl, int n_phase, const double *h_phases,
                      const int *h_reg_off, const double *h_regions, const soapgb_activity *act, double *d_temp,
                      double *d_bi, char *scratch, size_t scratch_bytes);
int integrate_device(soapgb_ctx *ctx, int form, int n, int n_eff, const double *d_wave, int grid, int n_phase,
                     const double *d_temp, const double *d_bi, const soapgb_maps &dm, const soapgb_cubes &dc,
                     double step, const soapgb_activity *act, void *d_flux, void *d_bconv, void *d_tot, int out_f32,
                     long long out_stride, int *d_cells, int *d_counts, char *fir_scratch, const FirPlanSizes &fp);
}  // namespace soapgb

// the FP32 form's deficits [spectrum][n] -> the FP64 raw output [spectrum][n_eff]
__global__ void k_widen_rows(long long n_rows, int n, int n_eff, const float *__restrict__ in, double *__restrict__ out) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_rows * n_eff) return;
    long long r = t / n_eff, i = t % n_eff;
    out[t] = soap_f32_to_f64(in[r * n + i]);
}

// Copies the `bytes` at src to every dst[k] (host memory), on up to eight host threads
// (one per 4 MiB of copies), each a contiguous share of the concatenated destinations.
static void host_replicate(const char *src, const std::vector<char *> &dst, size_t bytes) {
    const size_t total = bytes * dst.size();
    if (total == 0) return;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nt = (int)std::max<size_t>(1, std::min<size_t>({(size_t)8, (size_t)std::max(1u, hw / 2), total >> 22}));
    auto work = [&](int t) {
        const size_t a = total * t / nt, b = total * (t + 1) / nt;
        for (size_t o = a; o < b;) {
            const size_t d = o / bytes, off = o % bytes, len = std::min(bytes - off, b - o);
            memcpy(dst[d] + off, src + off, len);
            o += len;
        }
    };
    std::vector<std::thread> pool;
    int started = 1;
    try {
        for (int t = 1; t < nt; ++t, ++started) pool.emplace_back(work, t);
    } catch (...) {   // no thread to be had: the remaining shares on this one
    }
    for (int t = started; t < nt; ++t) work(t);
    work(0);
    for (auto &th : pool) th.join();
}

extern "C" int soapgb_phase_pipeline(soapgb_ctx *ctx, int form, int n, int n_eff, const double *wave,
                                     const soapgb_star *star, const soapgb_maps *maps, const soapgb_cubes *cubes,
                                     double step, const soapgb_activity *act, int n_phase, const double *phases,
                                     const int *reg_offsets, const double *regions, const double *quiet_sed,
                                     const double *quiet_norm, double sigma_v, double conv_step, double sentinel,
                                     int mem, double *lower, double *raw) {
    if (!ctx || !star || !maps || !cubes || !act) return SOAPGB_ERR_ARG;
    if (n < 3 || n_eff < 2 || n_eff > n || n_phase < 0 || !wave || !phases || !reg_offsets || !quiet_sed ||
        !quiet_norm || !lower || !(step > 0) || !(sigma_v > 0) || !(conv_step > 0) || cubes->n_mu < 1)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_phase_pipeline: bad arguments");
    if (form != SOAPGB_PLAIN64 && form != SOAPGB_FAST64 && form != SOAPGB_FAST32)
        return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_phase_pipeline: unknown form %d", form);
    if (n_phase == 0) return SOAPGB_OK;
    SOAP_DEVICE(ctx);
    bool host = (mem == SOAPGB_HOST);
    int grid = star->grid;
    long long gm = (long long)grid * grid;
    int n_mu = cubes->n_mu;
    // small descriptors on the host: read directly from host memory (no synchronisation,
    // so that a device-buffer call queues behind the previous one), or copied from device
    // memory with a synchronisation
    std::vector<int> h_off(n_phase + 1);
    std::vector<double> h_ph(n_phase);
    double w3[3];
    int rc0 = read_descriptor(ctx, h_off.data(), reg_offsets, sizeof(int) * (n_phase + 1));
    if (!rc0) rc0 = read_descriptor(ctx, h_ph.data(), phases, sizeof(double) * n_phase);
    if (rc0) return rc0;
    int n_rows = h_off[n_phase];
    if (h_off[0] != 0 || n_rows < 0) return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_phase_pipeline: bad reg_offsets");
    std::vector<double> h_reg(4 * (size_t)(n_rows > 0 ? n_rows : 1));
    if (n_rows > 0) {
        if (!regions) return set_error(ctx, SOAPGB_ERR_ARG, "soapgb_phase_pipeline: null regions");
        rc0 = read_descriptor(ctx, h_reg.data(), regions, sizeof(double) * 4 * n_rows);
        if (rc0) return rc0;
    }
    rc0 = wave_edges(ctx, mem, wave, n, n_eff, w3);
    if (rc0) return rc0;
    size_t cube_b = sizeof(double) * (size_t)n * n_mu;
    long long n_spec = 3LL * n_phase;
    // the collapsed forms build their per-phase cell lists from the regions' bounding
    // boxes (no G*G maps) when the grid allows; PLAIN64 integrates from the maps
    const bool collapsed = (form != SOAPGB_PLAIN64);
    const bool box_lists = collapsed && gm <= fir_box_lists_max_gm();
    Workspace ws(ctx);
    int s_wave = ws.add(host ? sizeof(double) * n : 0);
    int s_c[6];
    for (int q = 0; q < 4; ++q) s_c[q] = ws.add(host ? cube_b : 0);
    for (int q = 4; q < 6; ++q) s_c[q] = ws.add(host ? sizeof(double) * n : 0);
    int s_m[4];
    for (int q = 0; q < 3; ++q) s_m[q] = ws.add(host ? sizeof(double) * gm : 0);
    s_m[3] = ws.add(host ? sizeof(int) * gm : 0);
    int s_qs = ws.add(host ? sizeof(double) * n : 0);
    int s_qn = ws.add(host ? sizeof(double) * n : 0);
    int s_lower = ws.add(host ? sizeof(double) * (size_t)n_eff * n_spec : 0);
    size_t esz = (form == SOAPGB_FAST32) ? sizeof(float) : sizeof(double);
    int s_raw = ws.add(esz * (size_t)n * n_spec);                // deficits [p][type][n]
    int s_rawd = ws.add(form == SOAPGB_FAST32 && raw && host ? sizeof(double) * (size_t)n_eff * n_spec : 0);
    int s_temp = ws.add(box_lists ? 0 : sizeof(double) * gm * n_phase);
    int s_bi = ws.add(box_lists ? 0 : sizeof(double) * gm * n_phase);
    int s_cells = ws.add(collapsed ? 0 : sizeof(int) * gm * n_phase);
    int s_counts = ws.add(sizeof(int) * n_phase);
    // the region table and, after it, the small per-call lists (run / zero phases, zero
    // spectra, the convolution's row list): one upload
    const size_t pm_bytes = phase_maps_scratch_bytes(n_rows, n_phase);
    auto al256 = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t off_lists = al256(pm_bytes), off_zspec = off_lists + al256(sizeof(int) * n_phase);
    const size_t off_blist = off_zspec + al256((size_t)n_spec);
    const size_t small_bytes = off_blist + al256(sizeof(int) * ((size_t)n_spec + 2));
    int s_pm = ws.add(small_bytes);
    int s_ztmpl = ws.add(host && box_lists && form == SOAPGB_FAST32 ? sizeof(double) * 3 * (size_t)n_eff : 0);
    FirPlanSizes fp = fir_plan_sizes(form, n, n_mu, gm, true, n_phase);
    int s_fir = ws.add(fp.bytes);
    int s_res = ws.add(resolution_scratch_bytes(form, n, n_eff, (int)n_spec));
    int rc = ws.commit();
    if (rc) return rc;
    // Host buffers with a collapsed form: the cubes are copied in on the copy stream
    // while the geometry (cell order, lists, plans) is built; with FP32 the phases then
    // run in chunks, each chunk's spectra copied back on the copy stream while the next
    // chunk is computed.
    const bool overlap = host && collapsed;
    const bool chunked = overlap && form == SOAPGB_FAST32 && n_phase >= 2;
    int n_chunk = 1, per_chunk = n_phase;
    cudaStream_t cube_stream = ctx->stream;
    if (chunked) {
        n_chunk = std::min(n_phase, 8);
        per_chunk = (n_phase + n_chunk - 1) / n_chunk;
        n_chunk = (n_phase + per_chunk - 1) / per_chunk;
    }
    // call-long spans per stream (tracing only): from the call's start to each stream's
    // last operation
    std::unique_ptr<TraceScope> span_main, span_copy, span_d2h;
    if (overlap) {
        rc = copy_resources(ctx, n_chunk + 4);
        if (rc) return rc;
        span_main.reset(new TraceScope(ctx, "call_main"));
        span_copy.reset(new TraceScope(ctx, "call_copy", ctx->copy_stream));
        span_d2h.reset(new TraceScope(ctx, "call_d2h", ctx->d2h_stream));
        // the copy stream starts after the work already queued on the main stream
        SOAP_CUDA(ctx, cudaEventRecord(ctx->sync_events[0], ctx->stream));
        SOAP_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->sync_events[0], 0));
        cube_stream = ctx->copy_stream;
    }
#define STAGE(dst, src, bytes, slot)                                               \
    dst = (decltype(dst))stage_in(ctx, mem, src, bytes, ws.get<void>(slot), &rc); \
    if (rc) return rc;
#define STAGE_ON(stream, dst, src, bytes, slot)                                                       \
    if (host) {                                                                                       \
        SOAP_CUDA(ctx, cudaMemcpyAsync(ws.get<void>(slot), src, bytes, cudaMemcpyHostToDevice, stream)); \
        dst = (decltype(dst))ws.get<void>(slot);                                                      \
    } else {                                                                                          \
        dst = (decltype(dst))(src);                                                                   \
    }
    const double *d_wave;
    STAGE(d_wave, wave, sizeof(double) * n, s_wave);
    soapgb_cubes dc;
    dc.n_mu = n_mu;
    // small inputs first: copies share the host-to-device engine in issue order, so
    // the geometry's inputs must not queue behind the cubes
    STAGE(dc.spot_sed, cubes->spot_sed, sizeof(double) * n, s_c[4]);
    STAGE(dc.fac_sed, cubes->fac_sed, sizeof(double) * n, s_c[5]);
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
    const double *d_qs, *d_qn;
    STAGE(d_qs, quiet_sed, sizeof(double) * n, s_qs);
    STAGE(d_qn, quiet_norm, sizeof(double) * n, s_qn);
    char *d_raw = ws.get<char>(s_raw);
    int f32 = (form == SOAPGB_FAST32);
    double *d_temp = ws.get<double>(s_temp), *d_bi = ws.get<double>(s_bi);
    double *d_lower = host ? ws.get<double>(s_lower) : lower;
    const RegionPhase *d_table = nullptr;
    const int *d_roff = nullptr;
    // phases with a visible region are integrated; the others have no active cell
    std::vector<unsigned char> vis, zspec;
    std::vector<int> h_lists;   // run list, then zero list
    long long max_box = 0;      // most box cells of a phase
    int n_run = 0;
    std::vector<char> pack;   // image of the small-upload region
    int *d_lists = nullptr, *d_blist = nullptr;
    unsigned char *d_zspec = nullptr;
    int n_blist = -1;          // batches of the convolution's single chunk, when computed here
    if (box_lists) {
        rc = phase_table_device(ctx, grid, star->incl, n_phase, h_ph.data(), h_off.data(), h_reg.data(), act,
                                ws.get<char>(s_pm), pm_bytes, &d_table, &d_roff, &vis, &max_box, &pack);
        if (rc) return rc;
        for (int p = 0; p < n_phase; ++p)
            if (vis[p]) h_lists.push_back(p);
        n_run = (int)h_lists.size();
        for (int p = 0; p < n_phase; ++p)
            if (!vis[p]) h_lists.push_back(p);
        // spectra of the phases without a visible region are zero
        zspec.assign((size_t)n_spec, 0);
        for (int p = 0; p < n_phase; ++p) zspec[3 * p] = zspec[3 * p + 1] = zspec[3 * p + 2] = vis[p] ? 0 : 1;
        // the lists after the table, then one upload (a pageable source: staged by the
        // driver before the call returns)
        char *pm = ws.get<char>(s_pm);
        d_lists = (int *)(pm + off_lists);
        d_zspec = (unsigned char *)(pm + off_zspec);
        d_blist = (int *)(pm + off_blist);
        size_t used = off_zspec + (size_t)n_spec;
        std::vector<int> bl;
        if (!(host && collapsed) && form == SOAPGB_FAST32) {
            // device buffers: one chunk of all the spectra; its non-zero ones, the rows the
            // convolution takes
            for (long long q = 0; q < n_spec; ++q)
                if (!zspec[q]) bl.push_back((int)q);
            n_blist = (int)bl.size();
            used = off_blist + sizeof(int) * bl.size();
        }
        pack.resize(used, 0);
        memcpy(pack.data() + off_lists, h_lists.data(), sizeof(int) * n_phase);
        memcpy(pack.data() + off_zspec, zspec.data(), (size_t)n_spec);
        if (!bl.empty()) memcpy(pack.data() + off_blist, bl.data(), sizeof(int) * bl.size());
        SOAP_CUDA(ctx, cudaMemcpyAsync(pm, pack.data(), pack.size(), cudaMemcpyHostToDevice, ctx->stream));
    } else
        rc = phase_maps_device(ctx, grid, star->incl, n_phase, h_ph.data(), h_off.data(), h_reg.data(), act, d_temp,
                               d_bi, ws.get<char>(s_pm), pm_bytes);
    if (rc) return rc;
    // the cubes last, after every small upload (table, lists, flags) of the call
    {
        TraceScope ts(ctx, "h2d_cubes", cube_stream);
        STAGE_ON(cube_stream, dc.q_norm, cubes->q_norm, cube_b, s_c[0]);
        STAGE_ON(cube_stream, dc.q_sed, cubes->q_sed, cube_b, s_c[1]);
        STAGE_ON(cube_stream, dc.spot_norm, cubes->spot_norm, cube_b, s_c[2]);
        STAGE_ON(cube_stream, dc.fac_norm, cubes->fac_norm, cube_b, s_c[3]);
    }
    if (overlap) SOAP_CUDA(ctx, cudaEventRecord(ctx->sync_events[1], ctx->copy_stream));
#undef STAGE
#undef STAGE_ON
    if (collapsed) {
        FirPhaseArgs fa;
        fa.n = n;
        fa.n_eff = n_eff;
        fa.wave = d_wave;
        fa.cubes = &dc;
        fa.n_phase = n_phase;
        fa.temp = box_lists ? nullptr : d_temp;
        fa.bi = box_lists ? nullptr : d_bi;
        fa.table = d_table;
        fa.reg_off = d_roff;
        fa.grid = grid;
        fa.box_cap = box_lists ? fir_sorted_box_capacity(max_box) : 0;
        if (box_lists) {
            fa.run_list = d_lists;
            fa.zero_list = fa.run_list + n_run;
            fa.run_host = h_lists.data();
            fa.zero_host = h_lists.data() + n_run;
            fa.n_run = n_run;
            fa.n_zero = n_phase - n_run;
            // the FP32 resolution stage takes the zero phases as zero without reading
            // their rows; only the raw deficits, when wanted, need them written
            fa.zero_fill = (!f32 || raw) ? 1 : 0;
        }
        fa.delta = dm.delta;
        fa.limb = dm.limb;
        fa.lb = dm.lb;
        fa.region = dm.region;
        fa.gm = gm;
        fa.step = step;
        fa.act = act;
        fa.flux = d_raw + esz * n;
        fa.bconv = d_raw + esz * 2 * n;
        fa.tot = d_raw;
        fa.out_f32 = f32;
        fa.out_stride = 3LL * n;
        fa.lambda0 = w3[0];
        // The typed cubes and the convolution set-up (tap constants, FP64 base
        // convolutions) do not depend on the geometry stage (cell order, lists, plans),
        // which is latency-bound: they run beside it on the aux stream.  With host
        // buffers the convolution set-up needs only the small inputs, so it runs before
        // the cubes are in; the phases without a visible region then have their output
        // at once (the base alone, the same rows for every such phase), and it is copied
        // back on the d2h stream while the cubes are still coming in on the copy stream.
        const int n_zero = n_phase - n_run;
        const bool early_zero = host && f32 && box_lists && n_zero > 0;
        rc = aux_resources(ctx);
        if (rc) return rc;
        SOAP_CUDA(ctx, cudaEventRecord(ctx->aux_events[0], ctx->stream));
        SOAP_CUDA(ctx, cudaStreamWaitEvent(ctx->aux_stream, ctx->aux_events[0], 0));
        SOAP_CUDA(ctx, cudaStreamWaitEvent(ctx->geo_stream, ctx->aux_events[0], 0));
        Res32 R;
        {
            // host buffers: the convolution set-up first on the aux stream (its inputs
            // are in long before the cubes), then the typed cubes; device buffers: the
            // typed cubes on the aux stream and the convolution set-up on a second one,
            // both from the start, so that the FP64 base convolution overlaps the phase
            // lists (one block per phase, most SMs free) rather than the tile plans
            AuxScope aux(ctx);
            auto prepare = [&]() {
                return f32 ? resolution32_prepare(ctx, n, n_eff, (int)n_spec, d_wave, w3[0], w3[1], w3[2], d_qs, d_qn,
                                                  3, sigma_v, 50.0, conv_step, conv_step, sentinel,
                                                  ws.get<char>(s_res), R)
                           : SOAPGB_OK;
            };
            if (overlap) {
                rc = prepare();
            } else {
                rc = cuda_check(ctx, cudaStreamWaitEvent(ctx->aux2_stream, ctx->aux_events[0], 0), "set-up fork");
                if (!rc) {
                    AuxScope aux2(ctx, ctx->aux2_stream);
                    rc = prepare();
                    if (!rc) rc = cuda_check(ctx, cudaEventRecord(ctx->aux2_event, ctx->aux2_stream), "set-up join");
                }
            }
            if (!rc && early_zero) {
                rc = resolution32_zero_rows(ctx, R, 3, ws.get<double>(s_ztmpl));
                if (!rc) rc = cuda_check(ctx, cudaEventRecord(ctx->sync_events[2], ctx->aux_stream), "zero rows");
            }
            if (!rc && overlap) rc = cuda_check(ctx, cudaStreamWaitEvent(ctx->aux_stream, ctx->sync_events[1], 0),
                                                "cubes in");
            if (!rc) {
                fa.stage = FIR_STAGE_CUBES;
                rc = fir_phase(ctx, form, fa, ws.get<char>(s_fir), fp);
            }
            if (!rc) rc = cuda_check(ctx, cudaEventRecord(ctx->aux_events[2], ctx->aux_stream), "typed cubes");
            if (!rc && !overlap) rc = cuda_check(ctx, cudaStreamWaitEvent(ctx->aux_stream, ctx->aux2_event, 0), "set-up");
            if (!rc) rc = cuda_check(ctx, cudaEventRecord(ctx->aux_events[1], ctx->aux_stream), "aux join");
        }
        if (rc) return rc;
        // the zero phases' rows are all the same: one crosses the host link, and the host
        // copies it into the others while the visible phases are computed
        cudaEvent_t zero_ev = overlap ? ctx->sync_events[3 + n_chunk] : nullptr;
        if (early_zero) {
            SOAP_CUDA(ctx, cudaStreamWaitEvent(ctx->d2h_stream, ctx->sync_events[2], 0));
            TraceScope ts(ctx, "d2h_zero", ctx->d2h_stream);
            const double *tmpl = ws.get<double>(s_ztmpl);
            SOAP_CUDA(ctx, cudaMemcpyAsync(lower + (size_t)3 * h_lists[n_run] * n_eff, tmpl,
                                           sizeof(double) * 3 * n_eff, cudaMemcpyDeviceToHost, ctx->d2h_stream));
            SOAP_CUDA(ctx, cudaEventRecord(zero_ev, ctx->d2h_stream));
        }
        {
            // the geometry (lists, prefix sums, tile plans) is latency-bound and on the
            // critical path: on the high-priority stream, its blocks are dispatched ahead
            // of the aux stream's
            AuxScope geo(ctx, ctx->geo_stream);
            fa.stage = FIR_STAGE_GEOMETRY;
            rc = fir_phase(ctx, form, fa, ws.get<char>(s_fir), fp);
            if (!rc) rc = cuda_check(ctx, cudaEventRecord(ctx->geo_event, ctx->geo_stream), "geometry join");
        }
        if (rc) return rc;
        SOAP_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->geo_event, 0));
        // the integration needs the typed cubes; the convolution set-up is joined
        // before the first convolution, so with device buffers it runs on beside the
        // integration
        SOAP_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->aux_events[2], 0));
        if (f32) {
            bool joined = false;
            // phase range of the chunks: with the zero phases' rows already on their way,
            // only the visible phases' span is computed (unless the raw deficits are wanted)
            int c_lo = 0, c_hi = n_phase;
            if (early_zero && !raw) {
                c_lo = n_run > 0 ? h_lists[0] : 0;
                c_hi = n_run > 0 ? h_lists[n_run - 1] + 1 : 0;
            }
            const int span = c_hi - c_lo;
            const int nc = chunked ? std::max(1, std::min(n_chunk, span)) : 1;
            std::vector<int> cb;   // chunk c: phases [cb[c], cb[c + 1])
            if (span > 0) {
                const int per = (span + nc - 1) / nc;
                for (int c = 0; c < nc; ++c) cb.push_back(std::min(c_hi, c_lo + c * per));
                cb.push_back(c_hi);
            }
            for (int c = 0; c + 1 < (int)cb.size(); ++c) {
                const int p0 = cb[c], p1 = cb[c + 1];
                if (p0 >= p1) continue;
                fa.stage = FIR_STAGE_RUN;
                fa.l0 = p0;
                fa.l1 = p1;
                rc = fir_phase(ctx, form, fa, ws.get<char>(s_fir), fp);
                if (rc) return rc;
                if (!joined) {
                    SOAP_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->aux_events[1], 0));
                    joined = true;
                }
                rc = resolution32_run(ctx, R, (const float *)d_raw, n, 3 * p0, 3 * p1, d_lower, n_eff, nullptr,
                                      box_lists ? d_zspec : nullptr, box_lists ? zspec.data() : nullptr,
                                      early_zero ? ZeroRows::SKIP : ZeroRows::NORM,
                                      (n_blist >= 0 && p0 == 0 && p1 == n_phase) ? d_blist : nullptr, n_blist);
                if (rc) return rc;
                if (host) {
                    cudaEvent_t ev = ctx->sync_events[3 + c];
                    SOAP_CUDA(ctx, cudaEventRecord(ev, ctx->stream));
                    SOAP_CUDA(ctx, cudaStreamWaitEvent(ctx->d2h_stream, ev, 0));
                    TraceScope ts(ctx, "d2h_lower", ctx->d2h_stream);
                    // the chunk's phases, in runs; the zero phases' rows came from the template
                    for (int a = p0; a < p1;) {
                        if (early_zero && !vis[a]) {
                            ++a;
                            continue;
                        }
                        int b = a + 1;
                        while (b < p1 && !(early_zero && !vis[b])) ++b;
                        const size_t off = (size_t)3 * a * n_eff, cnt = (size_t)3 * (b - a) * n_eff;
                        SOAP_CUDA(ctx, cudaMemcpyAsync(lower + off, d_lower + off, sizeof(double) * cnt,
                                                       cudaMemcpyDeviceToHost, ctx->d2h_stream));
                        a = b;
                    }
                }
            }
            if (!joined) SOAP_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->aux_events[1], 0));
        } else {
            SOAP_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->aux_events[1], 0));
            fa.stage = FIR_STAGE_RUN;
            rc = fir_phase(ctx, form, fa, ws.get<char>(s_fir), fp);
            if (rc) return rc;
            rc = resolution_device(ctx, form, n, n_eff, (int)n_spec, d_wave, w3[0], w3[1], w3[2], d_raw, 0, n, d_qs,
                                   d_qn, 3, sigma_v, 50.0, conv_step, conv_step, sentinel, d_lower, n_eff, nullptr,
                                   ws.get<char>(s_res));
            if (rc) return rc;
            if (host)
                SOAP_CUDA(ctx, cudaMemcpyAsync(lower, d_lower, sizeof(double) * (size_t)n_eff * n_spec,
                                               cudaMemcpyDeviceToHost, ctx->stream));
        }
        if (raw) {
            long long tot_el = (long long)n_spec * n_eff;
            cudaMemcpyKind k = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
            if (f32) {
                double *dst = host ? ws.get<double>(s_rawd) : raw;
                SOAP_TRACED(ctx, "widen", k_widen_rows<<<grid_for(ctx, tot_el, 256), 256, 0, ctx->stream>>>(
                                              n_spec, n, n_eff, (const float *)d_raw, dst));
                SOAP_LAUNCHED(ctx);
                if (host)
                    SOAP_CUDA(ctx, cudaMemcpyAsync(raw, dst, sizeof(double) * tot_el, k, ctx->stream));
            } else {
                SOAP_CUDA(ctx, cudaMemcpy2DAsync(raw, sizeof(double) * n_eff, d_raw, sizeof(double) * n,
                                                 sizeof(double) * n_eff, n_spec, k, ctx->stream));
            }
        }
        if (!host) return SOAPGB_OK;
        if (early_zero && n_zero > 1) {
            SOAP_CUDA(ctx, cudaEventSynchronize(zero_ev));
            std::vector<char *> dst;
            for (int q = 1; q < n_zero; ++q) dst.push_back((char *)(lower + (size_t)3 * h_lists[n_run + q] * n_eff));
            host_replicate((const char *)(lower + (size_t)3 * h_lists[n_run] * n_eff), dst,
                           sizeof(double) * 3 * (size_t)n_eff);
        }
        span_main.reset();
        span_copy.reset();
        span_d2h.reset();
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->copy_stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->d2h_stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return check_status(ctx, "soapgb_phase_pipeline");
    }
    // PLAIN64: deficits in [phase][tot, flux, bconv][n] from the maps
    rc = integrate_device(ctx, form, n, n_eff, d_wave, grid, n_phase, d_temp, d_bi, dm, dc, step, act,
                          d_raw + esz * n /* flux */, d_raw + esz * 2 * n /* bconv */, d_raw /* tot */, 0, 3LL * n,
                          ws.get<int>(s_cells), ws.get<int>(s_counts), ws.get<char>(s_fir), fp);
    if (rc) return rc;
    rc = resolution_device(ctx, form, n, n_eff, (int)n_spec, d_wave, w3[0], w3[1], w3[2], d_raw, 0, n, d_qs, d_qn, 3,
                           sigma_v, 50.0, conv_step, conv_step, sentinel, d_lower, n_eff, nullptr, ws.get<char>(s_res));
    if (rc) return rc;
    if (raw) {
        cudaMemcpyKind k = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
        SOAP_CUDA(ctx, cudaMemcpy2DAsync(raw, sizeof(double) * n_eff, d_raw, sizeof(double) * n,
                                         sizeof(double) * n_eff, n_spec, k, ctx->stream));
    }
    if (host) {
        SOAP_CUDA(ctx, cudaMemcpyAsync(lower, d_lower, sizeof(double) * (size_t)n_eff * n_spec, cudaMemcpyDeviceToHost, ctx->stream));
        SOAP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return host ? check_status(ctx, "soapgb_phase_pipeline") : SOAPGB_OK;
}
