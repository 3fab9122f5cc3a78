// serve.cu -- continuous-batching query server over device-resident graphs.
//
// Requests (BFS rows, BC over a source set, reachable-vertex counts) arrive from
// any host thread.  A worker thread keeps a FIFO of pending requests and a fixed
// set of slots (stream, workspace, pinned staging of the inputs).  Whenever a
// slot is free it forms a batch from the oldest pending request and every later
// pending request it can share a launch with (up to max_batch sources; a larger
// request runs alone): BC requests of the same graph, or BFS and reachability
// requests of ANY graphs -- those run as one work-queue launch whose CTA groups
// take (graph, source block) items from a device counter -- and admits it if the
// batch's device footprint (engine workspace + rows)
// fits the HBM budget next to the batches already running, and launches it on
// the slot's stream with a persistent grid of 1/slots of the GPU, so batches of
// different slots overlap on the device.  Requests that arrive while batches
// run are admitted as slots and memory free up.  Per-request state lives on the
// device for the batch's lifetime: BFS requests own contiguous row ranges, BC
// requests own contiguous source ranges with their own bc vector
// (BcOptions::req_start), reachability requests own contiguous count ranges
// (counted in the kernel, no rows).  Each request's result is copied from the
// device straight into its own host buffer on the slot's stream.
// A request's result does not depend on its batch-mates: BFS rows and counts
// are exact; BC sums its sources in batch order, within 1e-12 of running alone.
#include "device_utils.cuh"
#include "gu_internal.h"

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <thread>
#include <unordered_map>
#include <unistd.h>

namespace gu {

int msbfs_ws_error(const Workspace &ws);
int bc_ws_error(const Workspace &ws);

using Clock = std::chrono::steady_clock;

struct SRequest {
    int64_t id = 0;
    int kind = 0;
    DeviceGraph *g = nullptr;
    std::vector<int32_t> src;
    void *out = nullptr;
    Clock::time_point t_submit, t_done;
    gu_status status = GU_OK;
    std::string err;
    bool done = false;
};

struct PinnedBuf {
    void *p = nullptr;
    size_t bytes = 0;
    void *get(size_t need)
    {
        if (need <= bytes && p) return p;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        GU_CUDA_CHECK(pinned_alloc(&p, need));
        bytes = need;
        return p;
    }
    ~PinnedBuf()
    {
        if (p) cudaFreeHost(p);
    }
};

struct Slot {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    Workspace ws, io;
    PinnedBuf stage;
    bool busy = false;
    int kind = 0;
    DeviceGraph *g = nullptr;
    std::vector<SRequest *> reqs;
    size_t need = 0;
    char *dres = nullptr;  // device results of the running batch, request after request
    bool copying = false;  // kernels done, results being copied out by the copier thread
    cudaError_t done_status = cudaSuccess;
    int touch_pending = 0;  // page-touch jobs of the batch's host buffers not yet done (tmu_)
    bool queued = false;       // the batch runs as a work-queue launch (ql), results at offs
    MsQueueLaunch ql;
    std::vector<size_t> offs;  // device result offset of each request (work-queue batches)
};

struct TouchJob {
    char *p;
    size_t bytes;
    Slot *slot;
};

class Server {
public:
    Server(size_t budget, int nslots, int max_batch) : budget_(budget), max_batch_(max_batch)
    {
        GU_CUDA_CHECK(cudaGetDevice(&device_));
        const int sms = device_sm_count(device_);
        sms_ = sms;
        nslots = std::max(1, std::min(nslots, 32));
        blocks_per_slot_ = std::max(1, 2 * sms / nslots);
        slots_.resize((size_t)nslots);
        for (Slot &s : slots_) {
            GU_CUDA_CHECK(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
            GU_CUDA_CHECK(cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming));
        }
        page_ = (size_t)sysconf(_SC_PAGESIZE);
        if (page_ < 4096) page_ = 4096;
        const unsigned hw = std::thread::hardware_concurrency();
        const int nt = (int)std::max(1u, std::min(12u, hw > 4 ? hw - 4 : 1u));
        for (int i = 0; i < nt; ++i) touchers_.emplace_back([this] { touch_loop(); });
        worker_ = std::thread([this] { loop(); });
        copier_ = std::thread([this] { copy_loop(); });
    }

    ~Server()
    {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_work_.notify_all();
        if (worker_.joinable()) worker_.join();  // returns once every slot's results are out
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_copier_ = true;
        }
        cv_copy_.notify_all();
        if (copier_.joinable()) copier_.join();
        {
            std::lock_guard<std::mutex> lk(tmu_);
            stop_touch_ = true;
        }
        cv_touch_.notify_all();
        for (std::thread &t : touchers_) t.join();
        cudaSetDevice(device_);
        for (Slot &s : slots_) {
            if (s.st) cudaStreamSynchronize(s.st);
            s.ws.release();
            s.io.release();
            if (s.ev) cudaEventDestroy(s.ev);
            if (s.st) cudaStreamDestroy(s.st);
        }
    }

    int64_t submit(int kind, DeviceGraph *g, const int32_t *src, int32_t k, void *out)
    {
        if (kind < GU_QUERY_BFS || kind > GU_QUERY_REACH) throw gu_error(GU_ERR_INVALID_ARGUMENT, "unknown query kind");
        if (!g || k <= 0 || !src || !out) throw gu_error(GU_ERR_INVALID_ARGUMENT, "bad request");
        if (g->device != device_) throw gu_error(GU_ERR_INVALID_ARGUMENT, "graph lives on another device");
        for (int32_t i = 0; i < k; ++i)
            if (src[i] < 0 || src[i] >= g->n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "source vertex out of range");
        std::unique_ptr<SRequest> r(new SRequest());
        r->kind = kind;
        r->g = g;
        r->src.assign(src, src + k);
        r->out = out;
        r->t_submit = Clock::now();
        int64_t id;
        {
            std::lock_guard<std::mutex> lk(mu_);
            id = r->id = ++next_id_;
            pending_.push_back(r.get());
            all_[id] = std::move(r);
        }
        cv_work_.notify_all();
        return id;
    }

    gu_status wait(int64_t id, double timeout_s, double *latency, std::string &err)
    {
        std::unique_lock<std::mutex> lk(mu_);
        auto it = all_.find(id);
        if (it == all_.end()) throw gu_error(GU_ERR_INVALID_ARGUMENT, "unknown request id");
        SRequest *r = it->second.get();
        const auto pred = [&] { return r->done; };
        if (timeout_s < 0) cv_done_.wait(lk, pred);
        else if (!cv_done_.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return GU_ERR_PENDING;
        if (latency) *latency = std::chrono::duration<double>(r->t_done - r->t_submit).count();
        const gu_status st = r->status;
        err = r->err;
        all_.erase(it);
        return st;
    }

    void stats(int64_t *completed, int64_t *batches, double *p50, double *p99, double *mean_batch)
    {
        std::lock_guard<std::mutex> lk(mu_);
        if (completed) *completed = completed_;
        if (batches) *batches = batches_;
        std::vector<double> l = latencies_;
        std::sort(l.begin(), l.end());
        auto pct = [&](double p) {
            if (l.empty()) return 0.0;
            size_t i = (size_t)std::ceil(p * (double)l.size()) - 1;
            return l[std::min(i, l.size() - 1)];
        };
        if (p50) *p50 = pct(0.50);
        if (p99) *p99 = pct(0.99);
        if (mean_batch) *mean_batch = batches_ ? (double)batched_reqs_ / (double)batches_ : 0.0;
    }

private:
    size_t row_bytes(const SRequest *r) const
    {
        if (r->kind == GU_QUERY_BFS) return r->src.size() * (size_t)r->g->n * sizeof(int32_t);
        if (r->kind == GU_QUERY_BC) return (size_t)r->g->n * sizeof(double);
        return r->src.size() * sizeof(long long);
    }

    size_t batch_need(int kind, const DeviceGraph &g, int32_t k, int nreq, size_t out_bytes) const
    {
        size_t ws = kind == GU_QUERY_BC ? bc_workspace_bytes(g, k, 0, true) : msbfs_workspace_bytes(g, k);
        size_t io = (size_t)k * 4 + (size_t)(nreq + 1) * 4 + 1024 + out_bytes;
        return ws + io;
    }

    size_t held_except(const Slot *self) const
    {
        size_t h = 0;
        for (const Slot &s : slots_)
            if (&s != self) h += s.ws.bytes + s.io.bytes;
        return h;
    }

    void finish(SRequest *r, gu_status st, const std::string &err)
    {
        r->status = st;
        r->err = err;
        r->t_done = Clock::now();
        r->done = true;
        ++completed_;
        latencies_.push_back(std::chrono::duration<double>(r->t_done - r->t_submit).count());
    }

    // Forms and launches a batch on slot s (mu_ held).  Returns true if launched.
    bool try_launch(Slot &s)
    {
        if (pending_.empty()) return false;
        SRequest *head = pending_.front();
        std::vector<SRequest *> batch{head};
        int32_t k = (int32_t)head->src.size();
        size_t out_bytes = row_bytes(head);
        const bool search = head->kind != GU_QUERY_BC;  // BFS rows and reachable counts share launches
        bool multi = false;
        for (size_t i = 1; i < pending_.size() && k < max_batch_; ++i) {
            SRequest *r = pending_[i];
            if (search ? r->kind == GU_QUERY_BC : (r->g != head->g || r->kind != head->kind)) continue;
            if (k + (int64_t)r->src.size() > max_batch_) continue;
            batch.push_back(r);
            k += (int32_t)r->src.size();
            out_bytes += row_bytes(r);
            multi |= r->g != head->g || r->kind != head->kind;
        }
        DeviceGraph &g = *head->g;
        size_t need = batch_need(head->kind, g, k, (int)batch.size(), out_bytes);
        std::vector<MsQueueRequest> qreqs;
        if (multi) {  // work-queue launch: its own workspace plan, outputs at 256-byte offsets
            qreqs.resize(batch.size());
            for (size_t i = 0; i < batch.size(); ++i) {
                qreqs[i].g = batch[i]->g;
                qreqs[i].sources = reinterpret_cast<const int32_t *>(1);  // placeholders: only sizes are planned
                qreqs[i].k = (int32_t)batch[i]->src.size();
                qreqs[i].ld = batch[i]->g->n;
                if (batch[i]->kind == GU_QUERY_BFS) qreqs[i].dist = reinterpret_cast<int32_t *>(1);
                else qreqs[i].reach = reinterpret_cast<unsigned long long *>(1);
            }
            out_bytes = 0;
            for (SRequest *r : batch) out_bytes += (row_bytes(r) + 255) / 256 * 256;
            need = msbfs_queue_plan(qreqs, sms_, blocks_per_slot_).bytes + (size_t)k * 4 + 1024 +
                   out_bytes;
        }
        if (held_except(&s) + std::max(need, s.ws.bytes + s.io.bytes) > budget_) {
            for (Slot &o : slots_)  // give back memory idle slots hold
                if (!o.busy && &o != &s) {
                    o.ws.release();
                    o.io.release();
                }
            s.ws.release();
            s.io.release();
            if (held_except(&s) + need > budget_) {
                bool any_busy = false;
                for (Slot &o : slots_) any_busy |= o.busy;
                if (any_busy) return false;  // wait for memory
                for (SRequest *r : batch) {  // can never fit
                    pending_.erase(std::find(pending_.begin(), pending_.end(), r));
                    finish(r, GU_ERR_CAPACITY, "request needs " + std::to_string(need) + " bytes of HBM, budget is " +
                                                   std::to_string(budget_));
                }
                cv_done_.notify_all();
                return false;
            }
        }
        for (SRequest *r : batch) pending_.erase(std::find(pending_.begin(), pending_.end(), r));
        try {
            if (multi) launch_queue(s, batch, k, out_bytes);
            else launch(s, head->kind, g, batch, k, out_bytes);
        } catch (const gu_error &e) {
            for (SRequest *r : batch) finish(r, e.code, e.what());
            cv_done_.notify_all();
            s.busy = false;
            return false;
        }
        s.need = need;
        ++batches_;
        batched_reqs_ += (int64_t)batch.size();
        return true;
    }

    void launch(Slot &s, int kind, DeviceGraph &g, const std::vector<SRequest *> &batch, int32_t k, size_t out_bytes)
    {
        GU_CUDA_CHECK(cudaSetDevice(device_));
        const int nreq = (int)batch.size();
        // pinned staging of the inputs: sources | request offsets
        const size_t src_b = ((size_t)k * 4 + 255) / 256 * 256;
        const size_t off_b = ((size_t)(nreq + 1) * 4 + 255) / 256 * 256;
        char *stage = (char *)s.stage.get(src_b + off_b + 256);
        int32_t *hs = reinterpret_cast<int32_t *>(stage);
        int32_t *hoff = reinterpret_cast<int32_t *>(stage + src_b);
        int32_t pos = 0;
        for (int i = 0; i < nreq; ++i) {
            hoff[i] = pos;
            std::memcpy(hs + pos, batch[i]->src.data(), batch[i]->src.size() * sizeof(int32_t));
            pos += (int32_t)batch[i]->src.size();
        }
        hoff[nreq] = pos;
        // device io: sources | offsets | outputs (BFS rows, bc vectors or reachable counts)
        const size_t res_b = (out_bytes + 255) / 256 * 256;
        char *io = (char *)s.io.get(src_b + off_b + res_b + 256);
        int32_t *dsrc = reinterpret_cast<int32_t *>(io);
        int32_t *doff = reinterpret_cast<int32_t *>(io + src_b);
        char *dres = io + src_b + off_b;
        GU_CUDA_CHECK(cudaMemcpyAsync(dsrc, hs, src_b + off_b, cudaMemcpyHostToDevice, s.st));
        {
            std::lock_guard<std::mutex> glk(g.mu);  // lazily built graph-side structures
            if (kind == GU_QUERY_BC) {
                BcOptions o;
                o.ws = &s.ws;
                o.max_blocks = blocks_per_slot_;
                o.timed = false;
                o.req_start = doff;
                o.nreq = nreq;
                launch_bc(g, dsrc, k, o, reinterpret_cast<double *>(dres), nullptr, nullptr, nullptr, g.n, true, s.st);
            } else {
                MsOptions o;
                o.variant = GU_BFS_AUTO;
                o.ws = &s.ws;
                o.max_blocks = blocks_per_slot_;
                o.timed = false;
                if (kind == GU_QUERY_REACH) {  // counts in the kernel, no rows
                    GU_CUDA_CHECK(cudaMemsetAsync(dres, 0, out_bytes, s.st));
                    o.reach = reinterpret_cast<unsigned long long *>(dres);
                    launch_msbfs(g, dsrc, k, nullptr, g.n, o, s.st, nullptr);
                } else {
                    launch_msbfs(g, dsrc, k, reinterpret_cast<int32_t *>(dres), g.n, o, s.st, nullptr);
                }
            }
        }
        s.dres = dres;
        s.queued = false;
        start_batch(s, kind, g, batch, out_bytes);
    }

    // Work-queue batch: BFS and reachability requests of several graphs in one
    // launch; request i's result at s.offs[i] (256-byte aligned) in the device io.
    void launch_queue(Slot &s, const std::vector<SRequest *> &batch, int32_t k, size_t out_bytes)
    {
        GU_CUDA_CHECK(cudaSetDevice(device_));
        const size_t src_b = ((size_t)k * 4 + 255) / 256 * 256;
        int32_t *hs = reinterpret_cast<int32_t *>(s.stage.get(src_b + 256));
        char *io = (char *)s.io.get(src_b + out_bytes + 256);
        int32_t *dsrc = reinterpret_cast<int32_t *>(io);
        char *dres = io + src_b;
        std::vector<MsQueueRequest> reqs(batch.size());
        s.offs.assign(batch.size(), 0);
        int32_t pos = 0;
        size_t off = 0;
        for (size_t i = 0; i < batch.size(); ++i) {
            const SRequest *r = batch[i];
            std::memcpy(hs + pos, r->src.data(), r->src.size() * sizeof(int32_t));
            MsQueueRequest &q = reqs[i];
            q.g = r->g;
            q.sources = dsrc + pos;
            q.k = (int32_t)r->src.size();
            q.ld = r->g->n;
            if (r->kind == GU_QUERY_BFS) q.dist = reinterpret_cast<int32_t *>(dres + off);
            else q.reach = reinterpret_cast<unsigned long long *>(dres + off);
            s.offs[i] = off;
            pos += q.k;
            off += (row_bytes(r) + 255) / 256 * 256;
        }
        GU_CUDA_CHECK(cudaMemcpyAsync(dsrc, hs, src_b, cudaMemcpyHostToDevice, s.st));
        s.ql = launch_msbfs_queue(reqs, s.ws, device_sm_count(device_), blocks_per_slot_, s.st);
        s.dres = dres;
        s.queued = true;
        start_batch(s, batch[0]->kind, *batch[0]->g, batch, out_bytes);
    }

    // Common tail of a launch: completion event, page touching of the requests'
    // host buffers, the slot's state (mu_ held).
    void start_batch(Slot &s, int kind, DeviceGraph &g, const std::vector<SRequest *> &batch, size_t out_bytes)
    {
        GU_CUDA_CHECK(cudaEventRecord(s.ev, s.st));
        {
            // touch the requests' host buffers while the batch runs, in pieces of
            // at least 4 MiB so every helper gets work on a large result
            std::lock_guard<std::mutex> tlk(tmu_);
            const size_t piece = std::max<size_t>((size_t)4 << 20, out_bytes / touchers_.size() + 1);
            for (SRequest *r : batch) {
                char *p = static_cast<char *>(r->out);
                const size_t b = row_bytes(r);
                for (size_t off = 0; off < b; off += piece) {
                    touch_q_.push_back({p + off, std::min(piece, b - off), &s});
                    ++s.touch_pending;
                }
            }
        }
        cv_touch_.notify_all();
        s.busy = true;
        s.kind = kind;
        s.g = &g;
        s.reqs = batch;
    }

    // Hands slot s's batch to the copier once its kernels are done (mu_ held).
    bool poll(Slot &s)
    {
        if (!s.busy || s.copying) return false;
        const cudaError_t q = cudaEventQuery(s.ev);
        if (q == cudaErrorNotReady) return false;
        s.done_status = q;
        s.copying = true;
        done_q_.push_back(&s);
        cv_copy_.notify_one();
        return true;
    }

    // Copies finished batches' results from the device straight into each
    // request's own host buffer, outside the server lock: on a coherent host
    // link a copy into pageable memory may run synchronously, and the worker
    // must keep launching meanwhile.
    void copy_loop()
    {
        cudaSetDevice(device_);
        std::unique_lock<std::mutex> lk(mu_);
        while (true) {
            cv_copy_.wait(lk, [&] { return !done_q_.empty() || stop_copier_; });
            if (done_q_.empty()) break;
            Slot &s = *done_q_.front();
            done_q_.pop_front();
            const std::vector<SRequest *> reqs = s.reqs;
            lk.unlock();
            gu_status st = GU_OK;
            std::string err;
            if (s.done_status != cudaSuccess) {
                st = GU_ERR_CUDA;
                err = cudaGetErrorString(s.done_status);
            } else {
                const int e = s.queued ? msbfs_queue_error(s.ws, s.ql)
                                       : s.kind == GU_QUERY_BC ? bc_ws_error(s.ws) : msbfs_ws_error(s.ws);
                if (e == DEV_ERR_BARRIER_TIMEOUT) {
                    st = GU_ERR_TIMEOUT;
                    err = "a device-side wait exceeded its limit";
                } else if (e != 0) {
                    st = e == 3 && s.kind == GU_QUERY_BC ? GU_ERR_CAPACITY : GU_ERR_INTERNAL;
                    err = "device reported error code " + std::to_string(e);
                }
            }
            {
                std::unique_lock<std::mutex> tlk(tmu_);
                cv_touched_.wait(tlk, [&] { return s.touch_pending == 0; });
            }
            if (st == GU_OK) {
                size_t off = 0;
                cudaError_t ce = cudaSuccess;
                for (size_t i = 0; i < reqs.size(); ++i) {
                    SRequest *r = reqs[i];
                    const size_t b = row_bytes(r);
                    const size_t o = s.queued ? s.offs[i] : off;
                    if (ce == cudaSuccess) ce = cudaMemcpyAsync(r->out, s.dres + o, b, cudaMemcpyDeviceToHost, s.st);
                    off += b;
                }
                if (ce == cudaSuccess) ce = cudaStreamSynchronize(s.st);
                if (ce != cudaSuccess) {
                    st = GU_ERR_CUDA;
                    err = cudaGetErrorString(ce);
                }
            }
            lk.lock();
            for (SRequest *r : reqs) finish(r, st, err);
            s.reqs.clear();
            s.copying = false;
            s.busy = false;
            cv_done_.notify_all();
            cv_work_.notify_all();
        }
    }

    // Helper thread: writes one byte of every page of a job's range (inside the
    // request's own output buffer, which the result copy overwrites later).
    void touch_loop()
    {
        std::unique_lock<std::mutex> lk(tmu_);
        while (true) {
            cv_touch_.wait(lk, [&] { return !touch_q_.empty() || stop_touch_; });
            if (touch_q_.empty()) return;
            const TouchJob j = touch_q_.front();
            touch_q_.pop_front();
            lk.unlock();
            volatile char *p = j.p;
            for (size_t off = 0; off < j.bytes; off += page_) p[off] = 0;
            if (j.bytes) p[j.bytes - 1] = 0;
            lk.lock();
            if (--j.slot->touch_pending == 0) cv_touched_.notify_all();
        }
    }

    void loop()
    {
        cudaSetDevice(device_);
        std::unique_lock<std::mutex> lk(mu_);
        while (true) {
            bool any_busy = false, progressed = false;
            for (Slot &s : slots_) progressed |= poll(s);
            for (Slot &s : slots_)
                if (!s.busy) progressed |= try_launch(s);
            for (Slot &s : slots_) any_busy |= s.busy;
            if (stop_ && !any_busy && pending_.empty()) break;
            if (!any_busy && !progressed) {
                cv_work_.wait_for(lk, std::chrono::milliseconds(50));
            } else if (!progressed) {
                lk.unlock();
                std::this_thread::sleep_for(std::chrono::microseconds(20));
                lk.lock();
            }
        }
    }

    size_t budget_;
    int max_batch_;
    int device_ = 0;
    int blocks_per_slot_ = 1;
    int sms_ = 1;
    std::vector<Slot> slots_;
    std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::deque<SRequest *> pending_;
    std::unordered_map<int64_t, std::unique_ptr<SRequest> > all_;
    int64_t next_id_ = 0, completed_ = 0, batches_ = 0, batched_reqs_ = 0;
    std::vector<double> latencies_;
    bool stop_ = false;
    std::thread worker_, copier_;
    std::condition_variable cv_copy_;
    std::deque<Slot *> done_q_;
    bool stop_copier_ = false;
    // page touching of the running batches' host buffers
    size_t page_ = 4096;
    std::vector<std::thread> touchers_;
    std::mutex tmu_;
    std::condition_variable cv_touch_, cv_touched_;
    std::deque<TouchJob> touch_q_;
    bool stop_touch_ = false;
};

Server *server_create(size_t budget, int nslots, int max_batch) { return new Server(budget, nslots, max_batch); }
void server_destroy(Server *s) { delete s; }
int64_t server_submit(Server *s, int kind, DeviceGraph *g, const int32_t *src, int32_t k, void *out)
{
    return s->submit(kind, g, src, k, out);
}
gu_status server_wait(Server *s, int64_t id, double timeout, double *latency, std::string &err)
{
    return s->wait(id, timeout, latency, err);
}
void server_stats(Server *s, int64_t *completed, int64_t *batches, double *p50, double *p99, double *mean_batch)
{
    s->stats(completed, batches, p50, p99, mean_batch);
}

}  // namespace gu
