/*
 * ref_shim.h -- force-included when compiling the reference graph-utils
 * example files that hold its CPU checkers (see oracle/build_ref.sh).
 *
 * Test infrastructure only.  The reference targets sm_35 and uses the pre-Volta
 * warp intrinsics __shfl/__ballot, which current CUDA no longer declares; the
 * device templates in its headers must still parse for the host checkers to
 * compile, so the unsynchronised forms are mapped onto the *_sync forms with a
 * full mask.  Three of the examples call parse(char*), an overload the
 * reference never defines; declaring it lets those files compile (their main()
 * is renamed and never called).
 */
#pragma once
#include <cuda_runtime.h>
#include <climits>
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 700
__device__ __forceinline__ int __shfl(int v, int l, int w = 32) { return __shfl_sync(0xffffffffu, v, l, w); }
__device__ __forceinline__ unsigned __ballot(int p) { return __ballot_sync(0xffffffffu, p); }
#endif
class host_graph;
host_graph parse(char *file);
