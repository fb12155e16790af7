// Active-voxel count without any device allocation.
//
// Some callers cannot allocate device memory at the time they need this
// count: host applications that hand the library a fixed device-memory
// budget up front and forbid third-party allocations afterwards, or code
// that must not risk an out-of-memory failure in the middle of a
// simulation.  For them the reduction below keeps its scratch in a
// file-scope device array instead of memory from cudaMalloc.
//
// Scratch: g_noalloc_scratch holds one partial count per CTA (at most
// NOALLOC_MAX_BLOCKS CTAs of NOALLOC_LEAVES_PER_BLOCK leaves each, so at most
// NOALLOC_MAX_LEAVES leaves per call) plus the final sum in its last entry:
// 65537 x 8 bytes = 512 KiB, resident on every GPU that loads this library
// until the process exits.  Every call overwrites the partials it uses and
// the final entry, so nothing needs clearing between calls; calls that
// overlap on the GPU (other streams, other threads) share the array and race.
//
// The array's name in host code is a host-side stand-in, not a device
// address.  Every call therefore looks up the device address with
// cudaGetSymbolAddress while the handle's device is current (a host-side
// lookup that allocates nothing); not caching it keeps a call correct after
// a device reset reloads the module and moves the array.
//
// The environment variable GBLS_NOALLOC_MAX_LEAVES, read by every call,
// lowers the leaf limit (never raises it), so tests can reach the rejection
// path and the exact limit on small grids.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <string>

namespace gbls {

constexpr int NOALLOC_LEAVES_PER_BLOCK = 32;
constexpr int NOALLOC_THREADS = NOALLOC_LEAVES_PER_BLOCK * 8;
constexpr int64_t NOALLOC_MAX_BLOCKS = 65536;
constexpr int64_t NOALLOC_MAX_LEAVES = NOALLOC_MAX_BLOCKS * NOALLOC_LEAVES_PER_BLOCK;

static __device__ __align__(256) unsigned long long g_noalloc_scratch[NOALLOC_MAX_BLOCKS + 1];

namespace {

// Per-CTA partial: popcounts of the active masks of NOALLOC_LEAVES_PER_BLOCK
// leaves (8 threads per leaf, one 64-bit mask word each).
__global__ void __launch_bounds__(NOALLOC_THREADS)
k_noalloc_partial(int64_t nleaf, const int32_t* slot, const uint64_t* am, unsigned long long* scratch) {
    const int64_t i = int64_t(blockIdx.x) * NOALLOC_THREADS + threadIdx.x;
    unsigned long long c = 0;
    if (i < nleaf * 8) c = __popcll(am[size_t(slot[i >> 3]) * 8 + (i & 7)]);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    __shared__ unsigned long long warp_sum[NOALLOC_THREADS / 32];
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        for (int w = 0; w < NOALLOC_THREADS / 32; ++w) s += warp_sum[w];
        scratch[blockIdx.x] = s;
    }
}

// One CTA sums the partials into scratch[NOALLOC_MAX_BLOCKS].
__global__ void __launch_bounds__(1024) k_noalloc_final(int nblocks, unsigned long long* scratch) {
    unsigned long long c = 0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) c += scratch[b];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    __shared__ unsigned long long warp_sum[32];
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) s += warp_sum[w];
        scratch[NOALLOC_MAX_BLOCKS] = s;
    }
}

int64_t leaf_limit() {
    const char* e = std::getenv("GBLS_NOALLOC_MAX_LEAVES");
    if (!e || !*e) return NOALLOC_MAX_LEAVES;
    const long long v = std::atoll(e);
    return (v < 0 || v > NOALLOC_MAX_LEAVES) ? NOALLOC_MAX_LEAVES : int64_t(v);
}

}  // namespace

// Count the active voxels of `nleaf` leaves (slot table `slot`, active
// masks `am`, both device arrays) on `stream` and store the count in *out.
// The current device must be the handle's.  Returns 0 on success (with the
// number of kernels launched in *launches), 1 for a grid over the leaf
// limit, 2 for a CUDA error; *err describes a failure.
int noalloc_count_active(int64_t nleaf, const int32_t* slot, const uint64_t* am, cudaStream_t stream,
                         int64_t* out, int* launches, std::string* err) {
    *launches = 0;
    const int64_t limit = leaf_limit();
    if (nleaf < 0 || nleaf > limit) {
        *err = "gbls_count_active_noalloc supports at most " + std::to_string(limit) + " leaves (got " +
               std::to_string(nleaf) + ")";
        return 1;
    }
    void* p = nullptr;
    const cudaError_t se = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (se != cudaSuccess) {
        *err = std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(se);
        return 2;
    }
    unsigned long long* scratch = static_cast<unsigned long long*>(p);
    if (nleaf == 0) {
        *out = 0;
        return 0;
    }
    const int nblocks = int((nleaf + NOALLOC_LEAVES_PER_BLOCK - 1) / NOALLOC_LEAVES_PER_BLOCK);
    k_noalloc_partial<<<nblocks, NOALLOC_THREADS, 0, stream>>>(nleaf, slot, am, scratch);
    k_noalloc_final<<<1, 1024, 0, stream>>>(nblocks, scratch);
    *launches = 2;
    cudaError_t e = cudaGetLastError();
    unsigned long long host = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&host, scratch + NOALLOC_MAX_BLOCKS, sizeof(host), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        *err = std::string("gbls_count_active_noalloc: ") + cudaGetErrorString(e);
        return 2;
    }
    *out = int64_t(host);
    return 0;
}

}  // namespace gbls
