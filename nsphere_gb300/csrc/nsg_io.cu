// nsg_io.cu -- the reference's particle files, read and written from the resident
// device state:
//   * the initial-conditions file of write_initial_conditions /
//     read_initial_conditions (nsphere.c:2386-2487): int32 npts, then npts records of
//     five doubles (r, v_r, ell, original index, mu);
//   * the all_particle_data snapshot stream (nsphere.c:1295-1324, written from the
//     time loop at nsphere.c:6452-6564): per snapshot, one 16-byte record per
//     particle in original-id order -- int32 rank (its index in the last sort),
//     float r, float v_r, float ell -- appended snapshot after snapshot.
// Records are packed and unpacked by kernels next to the state; the host side only
// moves contiguous blocks.  Initial-condition files stream through two pinned
// buffers so that file and PCIe/C2C transfers overlap.  Snapshots are written by a
// background thread from pinned slots while the next steps run: the record kernel
// runs on the context's stream and the copy on a separate stream.
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <mutex>
#include <thread>

#include "nsg_internal.cuh"

namespace nsg {

constexpr int64_t kIoChunk = int64_t(1) << 20;   // records per initial-condition chunk
constexpr int kSnapSlots = 2;                     // snapshots in flight

struct SnapRecord {
    int32_t rank;
    float r, v, l;
};
static_assert(sizeof(SnapRecord) == 16, "all_particle_data records are 16 bytes");

__global__ void k_unpack_init(const double *__restrict__ rec, int64_t count, int64_t off,
                              double *__restrict__ r, double *__restrict__ v, double *__restrict__ l,
                              double *__restrict__ id_d, double *__restrict__ aux)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count;
         k += (int64_t)gridDim.x * blockDim.x) {
        const double *q = rec + 5 * k;
        r[off + k] = q[0];
        v[off + k] = q[1];
        l[off + k] = q[2];
        id_d[off + k] = q[3];
        if (aux) aux[off + k] = q[4];
    }
}

__global__ void k_pack_init(double *__restrict__ rec, int64_t count, int64_t off, const double *__restrict__ r,
                            const double *__restrict__ v, const double *__restrict__ l,
                            const int32_t *__restrict__ id, const double *__restrict__ aux)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count;
         k += (int64_t)gridDim.x * blockDim.x) {
        double *q = rec + 5 * k;
        q[0] = r[off + k];
        q[1] = v[off + k];
        q[2] = l[off + k];
        q[3] = (double)id[off + k];
        q[4] = aux ? aux[off + k] : 0.0;
    }
}

// Record of particle `id`: its index in the last sort and its state there
// (nsphere.c:6466-6476: rank = inverse_map[id], values cast to float).
__global__ void k_pack_snapshot(SnapRecord *__restrict__ out, int64_t n, const int32_t *__restrict__ inv,
                                const double *__restrict__ r, const double *__restrict__ v,
                                const double *__restrict__ l)
{
    for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < n;
         id += (int64_t)gridDim.x * blockDim.x) {
        const int32_t p = inv[id];
        SnapRecord s;
        s.rank = p;
        s.r = (float)r[p];
        s.v = (float)v[p];
        s.l = (float)l[p];
        out[id] = s;
    }
}

// Background writer of one context's snapshot stream.
struct SnapWriter {
    FILE *f = nullptr;
    cudaStream_t copy = nullptr;
    SnapRecord *dev[kSnapSlots] = {};
    SnapRecord *host[kSnapSlots] = {};
    cudaEvent_t packed[kSnapSlots] = {}, copied[kSnapSlots] = {};
    bool busy[kSnapSlots] = {};
    int64_t count[kSnapSlots] = {};
    int64_t slot_cap[kSnapSlots] = {};   // records each slot holds
    int device = 0;
    int next = 0;
    std::deque<int> queue;           // slots waiting for the disk
    std::mutex mu;
    std::condition_variable cv;
    bool stop = false;
    bool failed = false;
    std::string err;
    std::thread th;

    void run()
    {
        cudaSetDevice(device);
        for (;;) {
            int s;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return stop || !queue.empty(); });
                if (queue.empty()) return;
                s = queue.front();
            }
            cudaError_t e = cudaEventSynchronize(copied[s]);
            bool ok = (e == cudaSuccess) &&
                      fwrite(host[s], sizeof(SnapRecord), (size_t)count[s], f) == (size_t)count[s];
            {
                std::lock_guard<std::mutex> lk(mu);
                queue.pop_front();
                busy[s] = false;
                if (!ok && !failed) {
                    failed = true;
                    err = e != cudaSuccess ? std::string("snapshot copy: ") + cudaGetErrorString(e)
                                           : std::string("snapshot write failed");
                }
            }
            cv.notify_all();
        }
    }
};

void snap_close(nsg_ctx *c)
{
    SnapWriter *w = c->snap;
    if (!w) return;
    {
        std::lock_guard<std::mutex> lk(w->mu);
        w->stop = true;
    }
    w->cv.notify_all();
    if (w->th.joinable()) w->th.join();
    if (w->f) fclose(w->f);
    for (int s = 0; s < kSnapSlots; s++) {
        cudaFree(w->dev[s]);
        cudaFreeHost(w->host[s]);
        if (w->packed[s]) cudaEventDestroy(w->packed[s]);
        if (w->copied[s]) cudaEventDestroy(w->copied[s]);
    }
    if (w->copy) cudaStreamDestroy(w->copy);
    delete w;
    c->snap = nullptr;
}

}  // namespace nsg

using namespace nsg;

extern "C" {

int nsg_write_init(nsg_ctx *c, const char *filename)
{
    if (!c || !filename) return set_err(c, NSG_EINVAL, "null context or file name");
    if (c->n <= 0) return set_err(c, NSG_ESTATE, "no state uploaded");
    if (c->n > 0x7fffffff) return set_err(c, NSG_EINVAL, "the file format holds at most 2^31-1 particles");
    FILE *f = fopen(filename, "wb");
    if (!f) return set_err(c, NSG_EINVAL, std::string("cannot open '") + filename + "' for writing");
    const int32_t npts = (int32_t)c->n;
    const int64_t chunk = c->n < kIoChunk ? c->n : kIoChunk;
    double *d_rec = nullptr, *h_rec[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t e = cudaMalloc((void **)&d_rec, (size_t)chunk * 40 * 2);
    for (int b = 0; b < 2 && e == cudaSuccess; b++) {
        e = cudaMallocHost((void **)&h_rec[b], (size_t)chunk * 40);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming);
    }
    bool io_ok = e == cudaSuccess && fwrite(&npts, sizeof(int32_t), 1, f) == 1;
    const int k = c->cur;
    const double *aux = c->p.carry_aux ? c->aux[k] : nullptr;
    int64_t pending_off = -1, pending_cnt = 0;
    int pb = 0;
    for (int64_t off = 0, it = 0; io_ok && e == cudaSuccess && off < c->n; off += chunk, it++) {
        const int b = (int)(it & 1);
        const int64_t cnt = (c->n - off < chunk) ? c->n - off : chunk;
        double *dr = d_rec + (size_t)b * chunk * 5;
        k_pack_init<<<grid_for(c, cnt, 256), 256, 0, c->stream>>>(dr, cnt, off, c->r[k], c->vr[k], c->ell[k],
                                                                   c->id[k], aux);
        e = cudaMemcpyAsync(h_rec[b], dr, (size_t)cnt * 40, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaEventRecord(ev[b], c->stream);
        // write the previous chunk while this one is packed and copied
        if (e == cudaSuccess && pending_off >= 0) {
            e = cudaEventSynchronize(ev[pb]);
            if (e == cudaSuccess) io_ok = fwrite(h_rec[pb], 40, (size_t)pending_cnt, f) == (size_t)pending_cnt;
        }
        pending_off = off;
        pending_cnt = cnt;
        pb = b;
    }
    if (io_ok && e == cudaSuccess && pending_off >= 0) {
        e = cudaEventSynchronize(ev[pb]);
        if (e == cudaSuccess) io_ok = fwrite(h_rec[pb], 40, (size_t)pending_cnt, f) == (size_t)pending_cnt;
    }
    if (fclose(f) != 0) io_ok = false;
    cudaStreamSynchronize(c->stream);
    cudaFree(d_rec);
    for (int b = 0; b < 2; b++) {
        cudaFreeHost(h_rec[b]);
        if (ev[b]) cudaEventDestroy(ev[b]);
    }
    if (e != cudaSuccess) return cuda_err(c, e, "write_init");
    if (!io_ok) return set_err(c, NSG_EINVAL, std::string("write to '") + filename + "' failed");
    return NSG_OK;
}

int nsg_read_init(nsg_ctx *c, const char *filename, int64_t expected_n)
{
    if (!c || !filename) return set_err(c, NSG_EINVAL, "null context or file name");
    FILE *f = fopen(filename, "rb");
    if (!f) return set_err(c, NSG_EINVAL, std::string("cannot open '") + filename + "' for reading");
    int32_t npts = 0;
    if (fread(&npts, sizeof(int32_t), 1, f) != 1 || npts <= 0) {
        fclose(f);
        return set_err(c, NSG_EINVAL, std::string("no particle count in '") + filename + "'");
    }
    if (expected_n >= 0 && expected_n != npts) {
        fclose(f);
        return set_err(c, NSG_EINVAL, "the file holds " + std::to_string(npts) + " particles, expected " +
                                          std::to_string(expected_n));
    }
    if (int rc = begin_upload(c, npts)) { fclose(f); return rc; }
    const int64_t n = npts, chunk = n < kIoChunk ? n : kIoChunk;
    double *d_rec = nullptr, *h_rec[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t e = cudaMalloc((void **)&d_rec, (size_t)chunk * 40 * 2);
    for (int b = 0; b < 2 && e == cudaSuccess; b++) {
        e = cudaMallocHost((void **)&h_rec[b], (size_t)chunk * 40);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming);
    }
    bool io_ok = true;
    double *aux = c->p.carry_aux ? c->aux[0] : nullptr;
    for (int64_t off = 0, it = 0; io_ok && e == cudaSuccess && off < n; off += chunk, it++) {
        const int b = (int)(it & 1);
        const int64_t cnt = (n - off < chunk) ? n - off : chunk;
        // the pinned buffer is free once the copy issued two chunks ago has finished
        if (it >= 2) e = cudaEventSynchronize(ev[b]);
        if (e != cudaSuccess) break;
        io_ok = fread(h_rec[b], 40, (size_t)cnt, f) == (size_t)cnt;
        if (!io_ok) break;
        double *dr = d_rec + (size_t)b * chunk * 5;
        e = cudaMemcpyAsync(dr, h_rec[b], (size_t)cnt * 40, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaEventRecord(ev[b], c->stream);
        k_unpack_init<<<grid_for(c, cnt, 256), 256, 0, c->stream>>>(dr, cnt, off, c->r[0], c->vr[0], c->ell[0],
                                                                     c->stage_d, aux);
    }
    fclose(f);
    int rc = NSG_OK;
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = cuda_err(c, e, "read_init");
    else if (!io_ok) rc = set_err(c, NSG_EINVAL, std::string("'") + filename + "' ends before its " +
                                                 std::to_string(npts) + " records");
    else rc = finish_upload_ids(c);
    cudaFree(d_rec);
    for (int b = 0; b < 2; b++) {
        cudaFreeHost(h_rec[b]);
        if (ev[b]) cudaEventDestroy(ev[b]);
    }
    if (rc != NSG_OK) c->n = 0;      // no half-read state is left resident
    return rc;
}

int nsg_snapshot_open(nsg_ctx *c, const char *filename, int append)
{
    if (!c || !filename) return set_err(c, NSG_EINVAL, "null context or file name");
    if (c->snap) return set_err(c, NSG_ESTATE, "a snapshot stream is already open");
    SnapWriter *w = new SnapWriter();
    w->device = c->device;
    w->f = fopen(filename, append ? "ab" : "wb");
    if (!w->f) {
        delete w;
        return set_err(c, NSG_EINVAL, std::string("cannot open '") + filename + "' for snapshots");
    }
    cudaError_t e = cudaStreamCreateWithFlags(&w->copy, cudaStreamNonBlocking);
    for (int s = 0; s < kSnapSlots && e == cudaSuccess; s++) {
        e = cudaEventCreateWithFlags(&w->packed[s], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->copied[s], cudaEventDisableTiming);
    }
    c->snap = w;
    if (e != cudaSuccess) {
        snap_close(c);
        return cuda_err(c, e, "snapshot stream setup");
    }
    w->th = std::thread([w] { w->run(); });
    return NSG_OK;
}

int nsg_snapshot(nsg_ctx *c)
{
    if (!c) return set_err(nullptr, NSG_EINVAL, "null context");
    SnapWriter *w = c->snap;
    if (!w) return set_err(c, NSG_ESTATE, "no snapshot stream open");
    if (c->n <= 0) return set_err(c, NSG_ESTATE, "no state uploaded");
    int s;
    {
        std::unique_lock<std::mutex> lk(w->mu);
        if (w->failed) return set_err(c, NSG_EINVAL, w->err);
        s = w->next;
        w->cv.wait(lk, [&] { return !w->busy[s]; });      // backpressure: the slot's last write is done
        w->busy[s] = true;
        w->next = (s + 1) % kSnapSlots;
    }
    cudaError_t e = cudaSuccess;
    if (w->slot_cap[s] < c->n) {
        cudaFree(w->dev[s]);
        cudaFreeHost(w->host[s]);
        w->dev[s] = nullptr;
        w->host[s] = nullptr;
        w->slot_cap[s] = 0;
        e = cudaMalloc((void **)&w->dev[s], (size_t)c->cap * sizeof(SnapRecord));
        if (e == cudaSuccess) e = cudaMallocHost((void **)&w->host[s], (size_t)c->cap * sizeof(SnapRecord));
        if (e == cudaSuccess) w->slot_cap[s] = c->cap;
    }
    if (e == cudaSuccess && !c->inv_valid) {
        // no sort since the upload: ranks are the positions of the uploaded order
        build_inv(c);
        c->inv_valid = true;
    }
    const int k = c->cur;
    if (e == cudaSuccess) {
        k_pack_snapshot<<<grid_for(c, c->n, 256), 256, 0, c->stream>>>(w->dev[s], c->n, c->inv, c->r[k], c->vr[k],
                                                                       c->ell[k]);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(w->packed[s], c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(w->copy, w->packed[s], 0);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(w->host[s], w->dev[s], (size_t)c->n * sizeof(SnapRecord), cudaMemcpyDeviceToHost,
                            w->copy);
    if (e == cudaSuccess) e = cudaEventRecord(w->copied[s], w->copy);
    if (e != cudaSuccess) {
        std::lock_guard<std::mutex> lk(w->mu);
        w->busy[s] = false;
        return cuda_err(c, e, "snapshot");
    }
    {
        std::lock_guard<std::mutex> lk(w->mu);
        w->count[s] = c->n;
        w->queue.push_back(s);
    }
    w->cv.notify_all();
    return NSG_OK;
}

int nsg_snapshot_close(nsg_ctx *c)
{
    if (!c) return set_err(nullptr, NSG_EINVAL, "null context");
    SnapWriter *w = c->snap;
    if (!w) return NSG_OK;
    bool failed;
    std::string err;
    {
        std::unique_lock<std::mutex> lk(w->mu);
        w->cv.wait(lk, [&] { return w->queue.empty(); });
        failed = w->failed;
        err = w->err;
    }
    const bool flushed = fflush(w->f) == 0;
    snap_close(c);
    if (failed) return set_err(c, NSG_EINVAL, err);
    if (!flushed) return set_err(c, NSG_EINVAL, "snapshot file flush failed");
    return NSG_OK;
}

}  // extern "C"
