// graph.cu -- the device-resident graph (replaces device_graph, device_graph.h:7-22
// and device_graph.cpp:3-14) and its workspace.
//
// Layout in HBM: R (n+1 int32), C (m int32), both from cudaMalloc (256-byte
// aligned); for directed graphs the in-edge CSR RT/CT (bottom-up levels pull
// over in-edges), for undirected graphs RT/CT alias R/C.  The COO source array F
// (device_graph's F) is built on the device on first use by the edge-parallel
// variant instead of being copied with every graph.
#include "device_utils.cuh"
#include "gu_internal.h"

#include <atomic>
#include <memory>
#include <mutex>

namespace gu {

// ---- allocation helpers with a host-side failure injector --------------------------
// After `after` more successful allocations, the next `count` fail.
static std::atomic<long long> g_fail_after{0}, g_fail_count{0};

void set_alloc_failures(long long after, long long count)
{
    g_fail_count.store(0);
    g_fail_after.store(after < 0 ? 0 : after);
    g_fail_count.store(count < 0 ? 0 : count);
}

static bool injected_failure()
{
    if (g_fail_count.load(std::memory_order_relaxed) <= 0) return false;
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (g_fail_count.load() <= 0) return false;
    if (g_fail_after.load() > 0) {
        g_fail_after.fetch_sub(1);
        return false;
    }
    g_fail_count.fetch_sub(1);
    return true;
}

cudaError_t dev_malloc(void **p, size_t bytes)
{
    if (injected_failure()) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    const cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) *p = nullptr;
    return e;
}

cudaError_t pinned_alloc(void **p, size_t bytes)
{
    if (injected_failure()) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    const cudaError_t e = cudaHostAlloc(p, bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) *p = nullptr;
    return e;
}

static std::atomic<unsigned long long> g_wait_ns{4ull * 1000ull * 1000ull * 1000ull};
unsigned long long wait_limit_ns() { return g_wait_ns.load(std::memory_order_relaxed); }
void set_wait_limit_ns(unsigned long long ns) { g_wait_ns.store(ns); }

// Diagnostic launch for gu_check_grid_barrier: every CTA but `absent` meets at two
// grid barriers; CTA `absent` leaves before its first arrival, so the others'
// first wait can only end by its limit.
__global__ void barrier_check_kernel(unsigned *bar, int *err, int absent, unsigned long long limit_ns, int *passed)
{
    unsigned epoch = 0;
    if ((int)blockIdx.x == absent) return;
    if (!grid_barrier(bar, err, epoch, limit_ns)) return;
    if (!grid_barrier(bar, err, epoch, limit_ns)) return;
    if (threadIdx.x == 0) atomicAdd(passed, 1);
}

int check_grid_barrier(int absent, unsigned long long limit_ns, cudaStream_t st, double *seconds)
{
    int dev = 0;
    GU_CUDA_CHECK(cudaGetDevice(&dev));
    const int blocks = device_sm_count(dev);
    if (absent < -1 || absent >= blocks)
        throw gu_error(GU_ERR_INVALID_ARGUMENT, "absent block must be -1 or in [0, " + std::to_string(blocks) + ")");
    struct Buf {
        int *p = nullptr;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        ~Buf()
        {
            if (p) cudaFree(p);
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
        }
    } b;
    GU_CUDA_CHECK(dev_malloc(reinterpret_cast<void **>(&b.p), 4 * sizeof(int)));
    GU_CUDA_CHECK(cudaEventCreate(&b.e0));
    GU_CUDA_CHECK(cudaEventCreate(&b.e1));
    GU_CUDA_CHECK(cudaMemsetAsync(b.p, 0, 4 * sizeof(int), st));
    unsigned *bar = reinterpret_cast<unsigned *>(b.p);
    int *err = b.p + 1, *passed = b.p + 2;
    void *params[] = {&bar, &err, &absent, &limit_ns, &passed};
    GU_CUDA_CHECK(cudaEventRecord(b.e0, st));
    GU_CUDA_CHECK(cudaLaunchCooperativeKernel((const void *)barrier_check_kernel, dim3(blocks), dim3(128), params, 0, st));
    GU_CUDA_CHECK(cudaEventRecord(b.e1, st));
    int h[4] = {0, 0, 0, 0};
    GU_CUDA_CHECK(cudaMemcpyAsync(h, b.p, sizeof(h), cudaMemcpyDeviceToHost, st));
    GU_CUDA_CHECK(cudaStreamSynchronize(st));
    float ms = 0.f;
    GU_CUDA_CHECK(cudaEventElapsedTime(&ms, b.e0, b.e1));
    if (seconds) *seconds = ms * 1e-3;
    if (h[1] == DEV_ERR_BARRIER_TIMEOUT)
        throw gu_error(GU_ERR_TIMEOUT, "a grid-barrier wait exceeded its limit (block " + std::to_string(absent) +
                                           " never arrived); " + std::to_string(h[2]) + " of " +
                                           std::to_string(blocks) + " blocks passed both barriers");
    if (h[1] != 0) throw gu_error(GU_ERR_INTERNAL, "device reported error code " + std::to_string(h[1]));
    if (h[2] != blocks - (absent >= 0 ? 1 : 0))
        throw gu_error(GU_ERR_INTERNAL, "grid barrier check: " + std::to_string(h[2]) + " of " +
                                            std::to_string(blocks) + " blocks passed");
    return blocks;
}

int device_sm_count(int device)
{
    int sms = 0;
    GU_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    return sms;
}

void *Workspace::get(size_t need)
{
    if (need <= bytes && ptr) return ptr;
    if (ptr) {
        GU_CUDA_CHECK(cudaDeviceSynchronize());
        GU_CUDA_CHECK(cudaFree(ptr));
        ptr = nullptr;
        bytes = 0;
    }
    size_t want = need + need / 8;
    cudaError_t e = dev_malloc(&ptr, want);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        ptr = nullptr;
        e = dev_malloc(&ptr, need);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            ptr = nullptr;
            throw gu_error(GU_ERR_OUT_OF_MEMORY, "workspace allocation of " + std::to_string(need) + " bytes failed");
        }
        want = need;
    }
    bytes = want;
    return ptr;
}

void Workspace::release()
{
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

void DeviceGraph::mark_start(cudaStream_t s)
{
    const int slot = ring_next;
    if (!ring_start[slot]) {
        GU_CUDA_CHECK(cudaEventCreate(&ring_start[slot]));
        GU_CUDA_CHECK(cudaEventCreate(&ring_stop[slot]));
    }
    ev_start = ring_start[slot];
    ev_stop = ring_stop[slot];
    GU_CUDA_CHECK(cudaEventRecord(ev_start, s));
}

void DeviceGraph::mark_stop(cudaStream_t s)
{
    GU_CUDA_CHECK(cudaEventRecord(ev_stop, s));
    timed = true;
    ring_next = (ring_next + 1) % LAUNCH_RING;
    if (ring_count < LAUNCH_RING) ++ring_count;
}

DeviceGraph::~DeviceGraph()
{
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    for (int i = 0; i < LAUNCH_RING; ++i) {
        if (ring_start[i]) cudaEventDestroy(ring_start[i]);
        if (ring_stop[i]) cudaEventDestroy(ring_stop[i]);
    }
    if (ctl_host) cudaFreeHost(ctl_host);
    if (copy_st) cudaStreamDestroy(copy_st);
    ws.release();
    io.release();
    if (F) cudaFree(F);
    for (void *p : extra_allocs) cudaFree(p);
    for (int32_t *p : {light, mid, wide, heavy})
        if (p) cudaFree(p);
    if (RT && RT != R) cudaFree(RT);
    if (CT && CT != C) cudaFree(CT);
    if (R) cudaFree(R);
    if (C) cudaFree(C);
    if (prev >= 0) cudaSetDevice(prev);
}

__global__ void coo_from_csr_kernel(const int32_t *__restrict__ R, int32_t n, int32_t *__restrict__ F)
{
    // one warp per vertex, lanes fill its CSR range
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (long long v = gw; v < n; v += nw) {
        const int32_t e1 = R[v + 1];
        for (int32_t e = R[v] + lane; e < e1; e += 32) F[e] = (int32_t)v;
    }
}

void ensure_coo(DeviceGraph &g, cudaStream_t stream)
{
    if (g.F || g.m == 0) return;
    GU_CUDA_CHECK(dev_malloc((void **)&g.F, sizeof(int32_t) * (size_t)g.m));
    g.bytes += sizeof(int32_t) * (size_t)g.m;
    coo_from_csr_kernel<<<g.sm_count * 4, 256, 0, stream>>>(g.R, g.n, g.F);
    GU_CUDA_CHECK(cudaGetLastError());
}

DeviceGraph *create_device_graph(const int32_t *R, const int32_t *C, int32_t n, int64_t m, bool directed,
                                 cudaStream_t stream)
{
    if (n < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "n must be >= 0");
    if (m < 0 || m > INT32_MAX) throw gu_error(GU_ERR_INVALID_ARGUMENT, "m must be in [0, INT32_MAX]");
    if (!R || (m > 0 && !C)) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null CSR array");
    if (R[0] != 0 || (int64_t)R[n] != m) throw gu_error(GU_ERR_INVALID_ARGUMENT, "R[0] must be 0 and R[n] must equal m");
    int32_t maxdeg = 0;
    for (int32_t v = 0; v < n; ++v) {
        const int32_t d = R[v + 1] - R[v];
        if (d < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "R must be non-decreasing");
        if (d > maxdeg) maxdeg = d;
    }
    for (int64_t e = 0; e < m; ++e)
        if (C[e] < 0 || C[e] >= n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "column index out of range");

    std::unique_ptr<DeviceGraph> g(new DeviceGraph());
    GU_CUDA_CHECK(cudaGetDevice(&g->device));
    g->sm_count = device_sm_count(g->device);
    g->n = n;
    g->m = m;
    g->directed = directed;
    g->max_degree = maxdeg;
    // Adjacency lists are stored by descending neighbour out-degree (ties by
    // id): search results are independent of list order, and bottom-up scans
    // meet the hubs, which most sources reach first, at the head of each list.
    std::vector<int32_t> outdeg((size_t)n);
    for (int32_t v = 0; v < n; ++v) outdeg[v] = R[v + 1] - R[v];
    std::vector<int32_t> Cs(C, C + m);
    sort_adjacency_by_key(R, Cs.data(), n, outdeg.data());
    g->host_R.assign(R, R + n + 1);
    GU_CUDA_CHECK(dev_malloc((void **)&g->R, sizeof(int32_t) * ((size_t)n + 1)));
    GU_CUDA_CHECK(dev_malloc((void **)&g->C, sizeof(int32_t) * (size_t)(m > 0 ? m : 1)));
    GU_CUDA_CHECK(cudaMemcpyAsync(g->R, R, sizeof(int32_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, stream));
    if (m > 0) GU_CUDA_CHECK(cudaMemcpyAsync(g->C, Cs.data(), sizeof(int32_t) * (size_t)m, cudaMemcpyHostToDevice, stream));
    g->bytes = sizeof(int32_t) * ((size_t)n + 1 + (size_t)m);
    if (directed) {
        HostGraph h;
        h.n = n;
        h.R.assign(R, R + n + 1);
        h.C.assign(C, C + m);
        HostGraph t = transpose(h);
        sort_adjacency_by_key(t.R.data(), t.C.data(), n, outdeg.data());
        g->host_RT = t.R;
        GU_CUDA_CHECK(dev_malloc((void **)&g->RT, sizeof(int32_t) * ((size_t)n + 1)));
        GU_CUDA_CHECK(dev_malloc((void **)&g->CT, sizeof(int32_t) * (size_t)(m > 0 ? m : 1)));
        GU_CUDA_CHECK(cudaMemcpyAsync(g->RT, t.R.data(), sizeof(int32_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, stream));
        if (m > 0) GU_CUDA_CHECK(cudaMemcpyAsync(g->CT, t.C.data(), sizeof(int32_t) * (size_t)m, cudaMemcpyHostToDevice, stream));
        GU_CUDA_CHECK(cudaStreamSynchronize(stream));  // t goes out of scope
        g->bytes *= 2;
    } else {
        g->RT = g->R;
        g->CT = g->C;
    }
    {
        // static lists of the bottom-up degree classes, by in-degree
        std::vector<int32_t> light, mid, wide, heavy;
        std::vector<int32_t> indeg((size_t)n, 0);
        if (directed) {
            for (int64_t e = 0; e < m; ++e) indeg[C[e]]++;
        } else {
            for (int32_t v = 0; v < n; ++v) indeg[v] = R[v + 1] - R[v];
        }
        for (int32_t v = 0; v < n; ++v) {
            if (indeg[v] > BU_HEAVY_DEGREE) heavy.push_back(v);
            else if (indeg[v] > BU_MID_DEGREE) wide.push_back(v);
            else if (indeg[v] > BU_LIGHT_DEGREE) mid.push_back(v);
            else if (indeg[v] > 0) light.push_back(v);
        }
        auto upload = [&](const std::vector<int32_t> &src, int32_t *&dst, int32_t &cnt) {
            cnt = (int32_t)src.size();
            if (src.empty()) return;
            GU_CUDA_CHECK(dev_malloc((void **)&dst, sizeof(int32_t) * src.size()));
            GU_CUDA_CHECK(cudaMemcpyAsync(dst, src.data(), sizeof(int32_t) * src.size(), cudaMemcpyHostToDevice, stream));
            g->bytes += sizeof(int32_t) * src.size();
        };
        upload(light, g->light, g->nlight);
        upload(mid, g->mid, g->nmid);
        upload(wide, g->wide, g->nwide);
        upload(heavy, g->heavy, g->nheavy);
        GU_CUDA_CHECK(cudaStreamSynchronize(stream));
    }
    return g.release();
}

}  // namespace gu
