// dag.cu -- reachable sets of every vertex of a DAG (the all-roots closure of
// graph-utils/dag_reachability.cpp:36-65), as per-vertex set sizes.
//
// The reference recurses from the roots with a std::set per vertex.  Here the
// closure is a multi-source search from every vertex at once: the batched
// engine (or the per-source one on low-degree graphs) counts the vertices each
// source reaches in the kernel, without distance rows; a vertex's reachable set
// excludes the vertex itself, as the reference's does.
#include "device_utils.cuh"
#include "gu_internal.h"

#include <algorithm>
#include <string>

namespace gu {

__global__ void iota_kernel(int32_t *v, int32_t n)
{
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

// counts[v] -= 1 (the source itself) and their sum into *total.
__global__ void reach_finish_kernel(long long *counts, int32_t n, unsigned long long *total)
{
    unsigned long long s = 0;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const long long c = counts[i] - 1;
        counts[i] = c;
        s += (unsigned long long)c;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL_MASK, s, o);
    if (lane_id() == 0 && s) atomicAdd(total, s);
}

void dag_reach(DeviceGraph &g, int64_t *counts, int64_t *total_host, cudaStream_t st)
{
    if (!g.directed) throw gu_error(GU_ERR_INVALID_ARGUMENT, "DAG reachability needs a directed graph");
    *total_host = 0;
    if (g.n == 0) return;
    char *io = (char *)g.io.get(256 + sizeof(int32_t) * (size_t)g.n);
    auto *total = reinterpret_cast<unsigned long long *>(io);
    int32_t *src = reinterpret_cast<int32_t *>(io + 256);
    const int blocks = std::min(g.sm_count * 8, (g.n + 255) / 256);
    GU_CUDA_CHECK(cudaMemsetAsync(total, 0, sizeof(unsigned long long), st));
    GU_CUDA_CHECK(cudaMemsetAsync(counts, 0, sizeof(int64_t) * (size_t)g.n, st));
    iota_kernel<<<blocks, 256, 0, st>>>(src, g.n);
    GU_CUDA_CHECK(cudaGetLastError());
    auto *cnt = reinterpret_cast<unsigned long long *>(counts);
    if (!(auto_engine(g, false) == AutoEngine::LOCAL && launch_local_bfs(g, src, g.n, nullptr, g.n, cnt, nullptr, st))) {
        GU_CUDA_CHECK(cudaMemsetAsync(counts, 0, sizeof(int64_t) * (size_t)g.n, st));
        MsOptions opt;
        opt.variant = GU_BFS_AUTO;
        opt.reach = cnt;
        launch_msbfs(g, src, g.n, nullptr, g.n, opt, st, nullptr);
        GU_CUDA_CHECK(cudaStreamSynchronize(st));
        int err = 0;
        msbfs_read_status(g, &err, nullptr, nullptr, nullptr);
        if (err == DEV_ERR_BARRIER_TIMEOUT) throw gu_error(GU_ERR_TIMEOUT, "a device-side wait exceeded its limit");
        if (err != 0) throw gu_error(GU_ERR_INTERNAL, "device reported error code " + std::to_string(err));
    }
    reach_finish_kernel<<<blocks, 256, 0, st>>>(reinterpret_cast<long long *>(counts), g.n, total);
    GU_CUDA_CHECK(cudaGetLastError());
    unsigned long long t = 0;
    GU_CUDA_CHECK(cudaMemcpyAsync(&t, total, sizeof(t), cudaMemcpyDeviceToHost, st));
    GU_CUDA_CHECK(cudaStreamSynchronize(st));
    *total_host = (int64_t)t;
}

}  // namespace gu
