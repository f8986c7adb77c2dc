// nsg_tune.cu -- autotuner of the step's launch shapes (no reference counterpart).
//
// Knobs (nsg::Tune): block size and blocks per SM of k_gather_level0, the bucket
// target of the near-sorted sort (sorted positions per splitter, a power of two),
// and blocks per SM of the level-parallel kernel.  nsg_autotune times candidate
// values on the resident state with the library's own CUDA-event profiler, one
// knob at a time (coordinate search), scoring each knob by the kernels it drives,
// then restores the state exactly as it was and keeps the fastest values.  The
// choice can be read back (nsg_tune_get) and stored by the caller keyed by N and
// GPU, and set again later (nsg_tune_set) without re-tuning.  Launch shapes change
// neither the arithmetic nor its order, so results do not depend on the tuning.
#include <cstdio>
#include <cstring>
#include <string>

#include "nsg_internal.cuh"

using namespace nsg;

namespace {

// A device copy of the current state and the device counters (status bits,
// point mass, histograms), so that trial steps leave no trace.
struct Snapshot {
    double *r = nullptr, *v = nullptr, *l = nullptr, *x = nullptr;
    int32_t *id = nullptr;
    DevCounters *ctr = nullptr;
    int cur = 0;
    int64_t steps = 0, launches = 0;
    double pm = 0.0;
};

void snap_free(Snapshot &s)
{
    cudaFree(s.r); cudaFree(s.v); cudaFree(s.l); cudaFree(s.id); cudaFree(s.x); cudaFree(s.ctr);
    s = Snapshot{};
}

int snap_take(nsg_ctx *c, Snapshot &s)
{
    const size_t b = (size_t)c->n * 8;
    cudaError_t e = cudaStreamSynchronize(c->side);
    if (e == cudaSuccess) e = cudaMalloc((void **)&s.r, b);
    if (e == cudaSuccess) e = cudaMalloc((void **)&s.v, b);
    if (e == cudaSuccess) e = cudaMalloc((void **)&s.l, b);
    if (e == cudaSuccess) e = cudaMalloc((void **)&s.id, (size_t)c->n * 4);
    if (e == cudaSuccess) e = cudaMalloc((void **)&s.ctr, sizeof(DevCounters));
    if (e == cudaSuccess && c->p.carry_aux) e = cudaMalloc((void **)&s.x, b);
    const int k = c->cur;
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.r, c->r[k], b, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.v, c->vr[k], b, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.l, c->ell[k], b, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.id, c->id[k], (size_t)c->n * 4, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.ctr, c->ctr, sizeof(DevCounters), cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess && s.x) e = cudaMemcpyAsync(s.x, c->aux[k], b, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { snap_free(s); return cuda_err(c, e, "tune snapshot"); }
    s.cur = k;
    s.steps = c->steps_done;
    s.launches = c->launches;
    s.pm = c->p.point_mass;
    return NSG_OK;
}

// Puts the snapshot back; the sort flags are reset so that the next step sorts
// from scratch (the radix path), exactly as after an upload.
int snap_put(nsg_ctx *c, const Snapshot &s)
{
    const size_t b = (size_t)c->n * 8;
    const int k = s.cur;
    cudaError_t e = cudaStreamSynchronize(c->side);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->r[k], s.r, b, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->vr[k], s.v, b, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->ell[k], s.l, b, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->id[k], s.id, (size_t)c->n * 4, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->ctr, s.ctr, sizeof(DevCounters), cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess && s.x) e = cudaMemcpyAsync(c->aux[k], s.x, b, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "tune restore");
    c->cur = k;
    c->state_epoch++;
    c->sorted = false;
    c->inv_valid = false;
    c->split_valid = false;
    c->steps_done = s.steps;
    c->launches = s.launches;
    c->p.point_mass = s.pm;
    return NSG_OK;
}

}  // namespace

extern "C" {

int nsg_tune_get(nsg_ctx *c, int32_t *vals, int count)
{
    if (!c || !vals || count < 4) return set_err(c, NSG_EINVAL, "tune needs 4 values");
    vals[0] = c->tune.gl0_threads; vals[1] = c->tune.gl0_bps;
    vals[2] = c->tune.bshift; vals[3] = c->tune.lanes_bps;
    return NSG_OK;
}

int nsg_tune_set(nsg_ctx *c, const int32_t *vals, int count)
{
    if (!c || !vals || count < 4) return set_err(c, NSG_EINVAL, "tune needs 4 values");
    const int th = vals[0], bps = vals[1], bs = vals[2], lb = vals[3];
    if ((th != 128 && th != 256 && th != 512) || bps < 1 || bps > 64 || bs < 8 || bs > 12 || lb < 1 || lb > 64)
        return set_err(c, NSG_EINVAL, "tune values out of range");
    const bool bucket_changed = (bs != c->tune.bshift);
    c->tune.gl0_threads = th; c->tune.gl0_bps = bps; c->tune.bshift = bs; c->tune.lanes_bps = lb;
    drop_graph(c);
    if (bucket_changed && c->n > 0) {
        // new bucket layout: re-derive the halo table; splitters come from the next radix sort
        std::vector<int64_t> hn((size_t)c->nseg);
        for (int h = 0; h < c->nseg; h++) hn[h] = c->h_seg_start[h + 1] - c->h_seg_start[h];
        if (int rc = set_halos(c, hn.data(), c->nseg)) return rc;
        c->split_valid = false;
    }
    return NSG_OK;
}

int nsg_autotune(nsg_ctx *c, int steps, char *report, int report_cap)
{
    if (!c) return set_err(nullptr, NSG_EINVAL, "null context");
    if (c->n <= 0) return set_err(c, NSG_ESTATE, "no state uploaded");
    if (c->mlp_collect) return set_err(c, NSG_ESTATE, "autotune while collecting scheduler data");
    if (steps < 1) steps = 1;
    Snapshot snap;
    if (int rc = snap_take(c, snap)) return rc;
    const Tune orig = c->tune;
    const bool was_profiling = c->profiling;
    std::string log = "{";
    char buf[256];

    // score = profiled milliseconds of the named kernels over `steps` steps (no
    // names: every kernel but the Levi-Civita chains, which no knob here changes)
    auto trial = [&](const Tune &t, std::initializer_list<const char *> names, double &score) -> int {
        int32_t v[4] = {t.gl0_threads, t.gl0_bps, t.bshift, t.lanes_bps};
        if (int rc = nsg_tune_set(c, v, 4)) return rc;
        if (int rc = nsg_step(c, 1)) return rc;          // warm (and refresh splitters)
        nsg_profile(c, 1);
        int rc = nsg_step(c, steps);
        nsg_kernel_stat st[64];
        int cnt = 0;
        if (!rc) rc = nsg_profile_read(c, st, 64, &cnt);
        nsg_profile(c, 0);
        if (rc) return rc;
        score = 0.0;
        for (int k = 0; k < cnt && k < 64; k++) {
            if (names.size() == 0) {
                if (strcmp(st[k].name, "levi_civita") != 0 && strcmp(st[k].name, "lc_late") != 0)
                    score += st[k].total_ms;
            }
            for (const char *nm : names)
                if (strcmp(st[k].name, nm) == 0) score += st[k].total_ms;
        }
        return snap_put(c, snap);
    };
    auto fail = [&](int rc) {
        int32_t v[4] = {orig.gl0_threads, orig.gl0_bps, orig.bshift, orig.lanes_bps};
        snap_put(c, snap);
        nsg_tune_set(c, v, 4);
        nsg_profile(c, was_profiling ? 1 : 0);
        snap_free(snap);
        return rc;
    };

    Tune best = orig;
    double s;
    // 1. bucket target of the near-sorted sort (9..11: sorted inside the kernel that
    //    consumes it; 12: bucket-sort kernel, then the gather), scored by the whole
    //    step beside the chains
    double bests = 1e300;
    log += "\"bucket_shift\":[";
    for (int bs : {10, 9, 11, 12}) {
        Tune t = best;
        t.bshift = bs;
        if (int rc = trial(t, {}, s)) return fail(rc);
        snprintf(buf, sizeof(buf), "%s[%d,%.4f]", log.back() == '[' ? "" : ",", bs, s / steps);
        log += buf;
        if (s < bests) { bests = s; best.bshift = bs; }
    }
    // 2. k_gather_level0 launch shape (the two-kernel path and the radix fallback's
    //    consumer; the fused kernels have one block per bucket)
    const int shapes[][2] = {{128, 16}, {256, 8}, {256, 4}, {512, 4}, {512, 2}};
    bests = 1e300;
    log += "],\"gather_level0\":[";
    for (auto &sh : shapes) {
        Tune t = best;
        t.gl0_threads = sh[0]; t.gl0_bps = sh[1];
        if (int rc = trial(t, {}, s)) return fail(rc);
        snprintf(buf, sizeof(buf), "%s[%d,%d,%.4f]", log.back() == '[' ? "" : ",", sh[0], sh[1], s / steps);
        log += buf;
        if (s < bests) { bests = s; best.gl0_threads = sh[0]; best.gl0_bps = sh[1]; }
    }
    // 3. level-parallel kernel grid
    bests = 1e300;
    log += "],\"levels\":[";
    for (int lb : {2, 4, 8}) {
        Tune t = best;
        t.lanes_bps = lb;
        if (int rc = trial(t, {}, s)) return fail(rc);
        snprintf(buf, sizeof(buf), "%s[%d,%.4f]", log.back() == '[' ? "" : ",", lb, s / steps);
        log += buf;
        if (s < bests) { bests = s; best.lanes_bps = lb; }
    }
    snprintf(buf, sizeof(buf), "],\"chosen\":[%d,%d,%d,%d]}", best.gl0_threads, best.gl0_bps, best.bshift,
             best.lanes_bps);
    log += buf;
    int32_t v[4] = {best.gl0_threads, best.gl0_bps, best.bshift, best.lanes_bps};
    int rc = nsg_tune_set(c, v, 4);
    nsg_profile(c, was_profiling ? 1 : 0);
    snap_free(snap);
    if (rc) return rc;
    if (report && report_cap > 0) {
        strncpy(report, log.c_str(), (size_t)report_cap - 1);
        report[report_cap - 1] = 0;
    }
    return NSG_OK;
}

}  // extern "C"
