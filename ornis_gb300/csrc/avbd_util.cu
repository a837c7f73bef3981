// avbd_util.cu — device-wide exclusive scan and stable LSD radix sort used by
// the broadphase (sorting AABB minima) and the pair-list builders (CSR offsets).
#include <cuda_runtime.h>

#include "avbd_kernels.h"

namespace avbd {

constexpr int SCAN_BLOCK = 1024;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// block-wide exclusive scan of one value per thread (blockDim == 1024)
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t inc = warp_incl_scan(v);
    if (lane == 31) warp_sums[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = warp_sums[lane];
        uint32_t si = warp_incl_scan(s);
        warp_sums[lane] = si - s;
        if (lane == 31 && total) *total = si;
    }
    __syncthreads();
    uint32_t r = inc - v + warp_sums[wid];
    __syncthreads();
    return r;
}

__global__ void k_scan_blocks(const uint32_t* in, uint32_t* out, size_t n, uint32_t* block_sums) {
    __shared__ uint32_t tot;
    size_t i = (size_t)blockIdx.x * SCAN_BLOCK + threadIdx.x;
    uint32_t v = i < n ? in[i] : 0u;
    uint32_t e = block_excl_scan(v, &tot);
    if (i < n) out[i] = e;
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

// single block: exclusive scan of the block sums (any count, looped)
__global__ void k_scan_sums(uint32_t* sums, size_t nb) {
    __shared__ uint32_t tot;
    uint32_t carry = 0;
    for (size_t base = 0; base < nb; base += SCAN_BLOCK) {
        size_t i = base + threadIdx.x;
        uint32_t v = i < nb ? sums[i] : 0u;
        uint32_t e = block_excl_scan(v, &tot);
        if (i < nb) sums[i] = e + carry;
        carry += tot;
        __syncthreads();
    }
}

__global__ void k_scan_add(uint32_t* out, size_t n, const uint32_t* block_sums) {
    size_t i = (size_t)blockIdx.x * SCAN_BLOCK + threadIdx.x;
    if (i < n) out[i] += block_sums[blockIdx.x];
}

size_t scan_tmp_words(size_t n) { return (n + SCAN_BLOCK - 1) / SCAN_BLOCK + 1; }

void scan_exclusive(const uint32_t* in, uint32_t* out, size_t n, uint32_t* tmp, cudaStream_t st) {
    if (n == 0) return;
    size_t nb = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
    k_scan_blocks<<<(unsigned)nb, SCAN_BLOCK, 0, st>>>(in, out, n, tmp);
    if (nb > 1) {
        k_scan_sums<<<1, SCAN_BLOCK, 0, st>>>(tmp, nb);
        k_scan_add<<<(unsigned)nb, SCAN_BLOCK, 0, st>>>(out, n, tmp);
    }
}

// ---- radix sort: 8-bit digits, tiles of RS_THREADS * RS_ITEMS keys ----------
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;

size_t radix_hist_words(size_t n) { return 256 * ((n + RS_TILE - 1) / RS_TILE) + 1; }

// hist layout: digit-major, [digit * ntiles + tile]
__global__ void k_rs_hist(const uint32_t* keys, size_t n, int shift, uint32_t* hist, int ntiles) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    size_t base = (size_t)blockIdx.x * RS_TILE;
    for (int it = 0; it < RS_ITEMS; it++) {
        size_t i = base + (size_t)it * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: items of a tile are processed in index order, RS_THREADS at
// a time; ranks inside a round come from warp match + per-warp digit counts.
__global__ void k_rs_scatter(const uint32_t* keys, const uint32_t* vals, uint32_t* okeys, uint32_t* ovals, size_t n,
                             int shift, const uint32_t* hist_scanned, int ntiles) {
    __shared__ uint32_t base_off[256];
    __shared__ uint32_t warp_cnt[RS_THREADS / 32][256];
    int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    base_off[tid] = hist_scanned[(size_t)tid * ntiles + blockIdx.x];
    size_t tile = (size_t)blockIdx.x * RS_TILE;
    for (int it = 0; it < RS_ITEMS; it++) {
        for (int w = 0; w < RS_THREADS / 32; w++) warp_cnt[w][tid] = 0;
        __syncthreads();
        size_t i = tile + (size_t)it * RS_THREADS + tid;
        bool valid = i < n;
        uint32_t k = valid ? keys[i] : 0u;
        uint32_t d = valid ? ((k >> shift) & 255u) : 256u;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        unsigned lt = (1u << lane) - 1u;
        uint32_t rank_w = __popc(peers & lt);
        if (valid && rank_w == 0) warp_cnt[wid][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t off = base_off[d] + rank_w;
            for (int w = 0; w < wid; w++) off += warp_cnt[w][d];
            okeys[off] = k;
            ovals[off] = vals[i];
        }
        __syncthreads();
        // advance the running offset of every digit by this round's count
        uint32_t add = 0;
        for (int w = 0; w < RS_THREADS / 32; w++) add += warp_cnt[w][tid];
        base_off[tid] += add;
        __syncthreads();
    }
}

int radix_pass(const uint32_t* keys, const uint32_t* vals, uint32_t* okeys, uint32_t* ovals, size_t n, int shift,
               uint32_t* hist, uint32_t* scan_tmp, cudaStream_t st) {
    int ntiles = (int)((n + RS_TILE - 1) / RS_TILE);
    if (n == 0) return 0;
    k_rs_hist<<<ntiles, RS_THREADS, 0, st>>>(keys, n, shift, hist, ntiles);
    scan_exclusive(hist, hist, (size_t)256 * ntiles, scan_tmp, st);
    k_rs_scatter<<<ntiles, RS_THREADS, 0, st>>>(keys, vals, okeys, ovals, n, shift, hist, ntiles);
    return ntiles;
}

void radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, size_t n,
                      uint32_t* hist, uint32_t* scan_tmp, cudaStream_t st) {
    if (n <= 1) return;
    int ntiles = (int)((n + RS_TILE - 1) / RS_TILE);
    uint32_t *ki = keys, *vi = vals, *ko = keys_alt, *vo = vals_alt;
    for (int pass = 0; pass < 4; pass++) {
        int shift = pass * 8;
        k_rs_hist<<<ntiles, RS_THREADS, 0, st>>>(ki, n, shift, hist, ntiles);
        scan_exclusive(hist, hist, (size_t)256 * ntiles, scan_tmp, st);
        k_rs_scatter<<<ntiles, RS_THREADS, 0, st>>>(ki, vi, ko, vo, n, shift, hist, ntiles);
        uint32_t* t = ki; ki = ko; ko = t;
        t = vi; vi = vo; vo = t;
    }
    // four passes: the result is back in (keys, vals)
}

}  // namespace avbd
