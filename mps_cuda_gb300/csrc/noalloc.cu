// mps_cell_sort_noalloc: the cell sort of the step (cell keys + stable radix sort) for callers
// that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is off limits -- inside a stream capture that a
// host application is recording, inside a plugin whose host owns the device allocator (a game
// engine or renderer that pools all GPU memory and forbids side allocations), or in a real-time
// loop where an allocation's implicit device synchronisation would stall the frame.  Such callers
// own their input and output buffers already; the only memory the sort needs beyond them is its
// ping-pong and histogram scratch, which here lives in one file-scope device array of fixed size
// that every GPU loading this library holds until the process exits (about 3.1 MB).
//
// Rules of use:
//  - n <= MPS_NOALLOC_MAX_PARTICLES (262144); larger inputs are rejected with MPS_E_INVALID.
//  - The first call on a device looks up the array's device address (cudaGetSymbolAddress) with
//    that device current; make that first call before any stream capture.
//  - All calls share the one array: calls that overlap on the GPU (different streams, or
//    different host threads on the same device) race on it and must be serialised by the caller.
//    Every byte of scratch that a call reads was written earlier in the same call (the histogram
//    is fully rewritten each digit pass), so the contents left by a previous call never leak in.
#include <cstdint>
#include <mutex>

#include "mps_c.h"
#include "mps_internal.cuh"

namespace mpsg {
namespace {

constexpr int kMax = MPS_NOALLOC_MAX_PARTICLES;
constexpr size_t kKeysBytes = size_t(kMax) * sizeof(unsigned long long);
constexpr size_t kValsBytes = size_t(kMax) * sizeof(unsigned int);
constexpr size_t kCountsBytes = size_t(256) * ((kMax + 4095) / 4096 + 1) * sizeof(unsigned int);  // + digit totals
constexpr size_t kScratchBytes = kKeysBytes + kValsBytes + kCountsBytes;

// Scratch of mps_cell_sort_noalloc: [tmp keys | tmp vals | digit histograms + totals].  In host code the
// name is only a stand-in; the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_base[64] = {};  // per-device address of g_noalloc_scratch

__global__ void k_noalloc_keys(const float4* __restrict__ pos4, int n, float ox, float oy, float oz, float inv,
                               int nx, int ny, int nz, unsigned long long* __restrict__ keys,
                               unsigned int* __restrict__ vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 x = pos4[i];
    const int cx = cell_coord(x.x, ox, inv, nx);
    const int cy = cell_coord(x.y, oy, inv, ny);
    const int cz = cell_coord(x.z, oz, inv, nz);
    keys[i] = grid_key(nx, ny, cx, cy, cz);
    vals[i] = unsigned(i);
}

}  // namespace
}  // namespace mpsg

using namespace mpsg;

extern "C" int mps_cell_sort_noalloc(const float* pos4, int64_t n, const float origin[3], float cell,
                                     const int32_t dims[3], uint64_t* keys_out, uint32_t* order_out, void* stream) {
    if (n < 0 || n > kMax) return MPS_E_INVALID;  // beyond the fixed scratch: rejected
    if (!origin || !dims || !(cell > 0.0f) || (n > 0 && (!pos4 || !keys_out || !order_out))) return MPS_E_INVALID;
    if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return MPS_E_INVALID;
    // pos4 is read as float4 (16-byte loads), keys and order with their natural alignment
    if (reinterpret_cast<uintptr_t>(pos4) % 16 != 0 || reinterpret_cast<uintptr_t>(keys_out) % 8 != 0 ||
        reinterpret_cast<uintptr_t>(order_out) % 4 != 0)
        return MPS_E_INVALID;
    const unsigned long long cells = cell_key_count(dims[0], dims[1], dims[2]);
    if (cells > (1ull << 40)) return MPS_E_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MPS_E_CUDA;
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_base[dev]) {
            if (cudaGetSymbolAddress(&g_base[dev], g_noalloc_scratch) != cudaSuccess) {
                g_base[dev] = nullptr;
                return MPS_E_CUDA;
            }
        }
        base = g_base[dev];
    }
    if (n == 0) return MPS_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    auto* tmp_keys = static_cast<unsigned long long*>(base);
    auto* tmp_vals = reinterpret_cast<unsigned int*>(static_cast<unsigned char*>(base) + kKeysBytes);
    auto* counts = reinterpret_cast<unsigned int*>(static_cast<unsigned char*>(base) + kKeysBytes + kValsBytes);
    const float inv = 1.0f / cell;
    auto* keys = reinterpret_cast<unsigned long long*>(keys_out);
    auto* vals = reinterpret_cast<unsigned int*>(order_out);
    // every launch's own status is checked (cudaLaunchKernelEx here, the same in the radix sort), so an
    // earlier, unrelated error pending in the calling thread is neither reported nor cleared
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(unsigned((n + 255) / 256));
    cfg.blockDim = dim3(256u);
    cfg.stream = s;
    if (cudaLaunchKernelEx(&cfg, k_noalloc_keys, reinterpret_cast<const float4*>(pos4), int(n), origin[0], origin[1],
                           origin[2], inv, dims[0], dims[1], dims[2], keys, vals) != cudaSuccess)
        return MPS_E_CUDA;
    int bits = 1;
    while ((1ull << bits) < cells) bits++;
    return radix_sort_pairs(keys, vals, tmp_keys, tmp_vals, counts, int(n), bits, 8, s) == cudaSuccess ? MPS_OK
                                                                                                       : MPS_E_CUDA;
}
