// Stable LSD radix sort of (64-bit cell key, 32-bit slot) pairs over the significant key bits
// only.  Replaces the thrust::sort_by_key of SpatialHash::UpdateHash (MPSSpatialHash.cu:69),
// whose stability fixes the within-cell order; this sort keeps the same stability guarantee.
//
// One pass per digit (digit_bits <= 8):
//   upsweep  : per-tile digit histogram (warp-aggregated shared atomics), digit-major counts
//   scan     : per digit, a warp scans that digit's row of tile counts (coalesced, all digits in
//              parallel); one block scans the 256 digit totals; the downsweep adds both
//   downsweep: per-warp stable ranks with __match_any_sync, cross-warp prefix per digit, scatter
// Tiles are 8 warps x 32 lanes x 16 items; each warp owns a contiguous run of 512 keys, so
// (warp, round, lane) order equals input order and the scatter is stable.
#include "mps_internal.cuh"

namespace mpsg {

namespace {
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kIpt = 16;
constexpr int kTile = kThreads * kIpt;
constexpr int kBins = 256;

__global__ void __launch_bounds__(kThreads) rs_upsweep(const unsigned long long* __restrict__ keys, int n,
                                                       int shift, unsigned int mask, int nblocks,
                                                       unsigned int* __restrict__ counts) {
    __shared__ unsigned int hist[kBins];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wbase = blockIdx.x * kTile + warp * 32 * kIpt;
#pragma unroll 4
    for (int r = 0; r < kIpt; ++r) {
        const int idx = wbase + r * 32 + lane;
        const bool valid = idx < n;
        const unsigned int d = valid ? unsigned((keys[idx] >> shift) & mask) : 0xffffffffu;
        const unsigned int peers = __match_any_sync(0xffffffffu, d);
        if (valid && lane == __ffs(peers) - 1) atomicAdd(&hist[d], unsigned(__popc(peers)));
    }
    __syncthreads();
    counts[threadIdx.x * nblocks + blockIdx.x] = hist[threadIdx.x];
}

// counts[d * nblocks + b] <- exclusive prefix over tiles b of digit d; totals[d] <- digit total.
__global__ void __launch_bounds__(kThreads) rs_scan_rows(unsigned int* __restrict__ counts, int nblocks,
                                                         unsigned int* __restrict__ totals) {
    const int lane = threadIdx.x & 31;
    const int digit = blockIdx.x * kWarps + (threadIdx.x >> 5);
    if (digit >= kBins) return;
    unsigned int* row = counts + size_t(digit) * size_t(nblocks);
    unsigned int run = 0;
    for (int base = 0; base < nblocks; base += 32) {
        const int idx = base + lane;
        const unsigned int v = idx < nblocks ? row[idx] : 0u;
        unsigned int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (idx < nblocks) row[idx] = run + incl - v;
        run += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) totals[digit] = run;
}

// totals[d] <- exclusive prefix over digits (one block of kBins threads).
__global__ void __launch_bounds__(kBins) rs_scan_digits(unsigned int* __restrict__ totals) {
    __shared__ unsigned int warp_sums[kBins / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned int v = totals[threadIdx.x];
    unsigned int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    unsigned int before = 0;
    for (int w = 0; w < warp; ++w) before += warp_sums[w];
    totals[threadIdx.x] = before + incl - v;
}

__global__ void __launch_bounds__(kThreads) rs_downsweep(const unsigned long long* __restrict__ kin,
                                                         const unsigned int* __restrict__ vin,
                                                         unsigned long long* __restrict__ kout,
                                                         unsigned int* __restrict__ vout, int n,
                                                         int shift, unsigned int mask, int nblocks,
                                                         const unsigned int* __restrict__ offsets,
                                                         const unsigned int* __restrict__ digit_base) {
    __shared__ unsigned int wcnt[kWarps][kBins];
    __shared__ unsigned int s_off[kBins];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) wcnt[w][threadIdx.x] = 0;
    s_off[threadIdx.x] = offsets[threadIdx.x * nblocks + blockIdx.x] + digit_base[threadIdx.x];
    __syncthreads();
    const int wbase = blockIdx.x * kTile + warp * 32 * kIpt;
    const unsigned int lt = (1u << lane) - 1u;
    unsigned long long k[kIpt];
    unsigned int v[kIpt];
    unsigned int rank[kIpt];
#pragma unroll
    for (int r = 0; r < kIpt; ++r) {
        const int idx = wbase + r * 32 + lane;
        const bool valid = idx < n;
        k[r] = valid ? kin[idx] : 0ull;
        v[r] = valid ? vin[idx] : 0u;
        const unsigned int d = valid ? unsigned((k[r] >> shift) & mask) : 0xffffffffu;
        const unsigned int peers = __match_any_sync(0xffffffffu, d);
        const unsigned int base = valid ? wcnt[warp][d] : 0u;
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] = base + unsigned(__popc(peers));
        __syncwarp();
        rank[r] = base + unsigned(__popc(peers & lt));
    }
    __syncthreads();
    {   // exclusive prefix over warps for digit threadIdx.x
        unsigned int run = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const unsigned int c = wcnt[w][threadIdx.x];
            wcnt[w][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kIpt; ++r) {
        const int idx = wbase + r * 32 + lane;
        if (idx < n) {
            const unsigned int d = unsigned((k[r] >> shift) & mask);
            const unsigned int dst = s_off[d] + wcnt[warp][d] + rank[r];
            kout[dst] = k[r];
            vout[dst] = v[r];
        }
    }
}
}  // namespace

// tile counts (digit-major) followed by the kBins digit totals
size_t radix_counts_size(int n) {
    const int nblocks = (n + kTile - 1) / kTile;
    return size_t(kBins) * size_t(nblocks > 0 ? nblocks : 1) + kBins;
}

// Launches one kernel and returns that launch's status (cudaLaunchKernelEx reports the launch
// itself, unlike cudaGetLastError, which would also return an earlier, unrelated error of the thread).
template <class... KArgs, class... Args>
static cudaError_t launch_checked(void (*k)(KArgs...), int grid, int block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(unsigned(grid));
    cfg.blockDim = dim3(unsigned(block));
    cfg.stream = s;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

cudaError_t radix_sort_pairs(unsigned long long* keys, unsigned int* vals, unsigned long long* keys_tmp,
                             unsigned int* vals_tmp, unsigned int* counts, int n, int bits, int digit_bits,
                             cudaStream_t s) {
    if (n <= 1 || bits <= 0) return cudaSuccess;
    if (digit_bits < 1 || digit_bits > 8) digit_bits = 8;
    const int nblocks = (n + kTile - 1) / kTile;
    const int passes = (bits + digit_bits - 1) / digit_bits;
    unsigned long long *ka = keys, *kb = keys_tmp;
    unsigned int *va = vals, *vb = vals_tmp;
    cudaError_t e = cudaSuccess;
    for (int p = 0; p < passes; ++p) {
        const int shift = p * digit_bits;
        const int nb = min(digit_bits, bits - shift);
        const unsigned int mask = (1u << nb) - 1u;
        unsigned int* totals = counts + size_t(kBins) * size_t(nblocks);
        if ((e = launch_checked(rs_upsweep, nblocks, kThreads, s, (const unsigned long long*)ka, n, shift, mask,
                                nblocks, counts)) != cudaSuccess)
            return e;
        if ((e = launch_checked(rs_scan_rows, kBins / kWarps, kThreads, s, counts, nblocks, totals)) != cudaSuccess)
            return e;
        if ((e = launch_checked(rs_scan_digits, 1, kBins, s, totals)) != cudaSuccess) return e;
        if ((e = launch_checked(rs_downsweep, nblocks, kThreads, s, (const unsigned long long*)ka,
                                (const unsigned int*)va, kb, vb, n, shift, mask, nblocks,
                                (const unsigned int*)counts, (const unsigned int*)totals)) != cudaSuccess)
            return e;
        unsigned long long* tk = ka; ka = kb; kb = tk;
        unsigned int* tv = va; va = vb; vb = tv;
    }
    if (ka != keys) {
        if ((e = cudaMemcpyAsync(keys, ka, size_t(n) * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s)) !=
            cudaSuccess)
            return e;
        e = cudaMemcpyAsync(vals, va, size_t(n) * sizeof(unsigned int), cudaMemcpyDeviceToDevice, s);
    }
    return e;
}

}  // namespace mpsg
