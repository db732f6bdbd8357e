// radix_sort.cuh -- stable LSD radix sort of (uint32 key, uint32 value)
// pairs, 4 bits per pass, for the per-step cell ordering of the particles.
//
// One pass = three kernels:
//   rs_count   each tile (256 threads x RS_ITEMS keys) counts its 16 digits
//              into hist[digit * ntiles + tile];
//   rs_scan    one CTA turns hist into exclusive offsets (digit-major, so
//              equal digits keep tile order);
//   rs_scatter each tile ranks its keys stably (per-thread digit counters,
//              block-wide scan over [digit][thread]) and writes them to
//              offset + rank.
// Keys of deleted particles are the largest key, so they sort to the end.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace plume {

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_BINS = 16;

__global__ void rs_count(const uint32_t* __restrict__ keys, int n, int shift,
                         uint32_t* __restrict__ hist, int ntiles) {
  __shared__ uint32_t cnt[RS_BINS];
  if (threadIdx.x < RS_BINS) cnt[threadIdx.x] = 0;
  __syncthreads();
  const int base = blockIdx.x * RS_TILE;
  for (int k = 0; k < RS_ITEMS; k++) {
    int idx = base + k * RS_THREADS + threadIdx.x;
    if (idx < n) atomicAdd(&cnt[(keys[idx] >> shift) & 0xF], 1u);
  }
  __syncthreads();
  if (threadIdx.x < RS_BINS) hist[threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

// exclusive scan of m = 16 * ntiles counters by one CTA of 1024 threads
__global__ void rs_scan(uint32_t* __restrict__ hist, int m) {
  __shared__ uint32_t part[1024];
  const int t = threadIdx.x;
  const int per = (m + 1023) / 1024;
  const int lo = t * per;
  const int hi = min(lo + per, m);
  uint32_t s = 0;
  for (int i = lo; i < hi; i++) s += hist[i];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    uint32_t v = (t >= off) ? part[t - off] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  uint32_t run = (t == 0) ? 0u : part[t - 1];
  for (int i = lo; i < hi; i++) {
    uint32_t v = hist[i];
    hist[i] = run;
    run += v;
  }
}

__global__ void rs_scatter(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                           uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int n,
                           int shift, const uint32_t* __restrict__ hist, int ntiles) {
  // counters[digit][thread] as 16-bit halves packed in 32-bit words
  __shared__ uint32_t cnt[RS_BINS * RS_THREADS];
  __shared__ uint32_t tile_off[RS_BINS];
  __shared__ uint32_t wsum[RS_THREADS / 32];
  const int t = threadIdx.x;
  const int base = blockIdx.x * RS_TILE + t * RS_ITEMS;  // blocked arrangement
  uint32_t k[RS_ITEMS], v[RS_ITEMS];
  int d[RS_ITEMS];
#pragma unroll
  for (int q = 0; q < RS_ITEMS; q++) {
    int idx = base + q;
    if (idx < n) {
      k[q] = keys_in[idx];
      v[q] = vals_in[idx];
      d[q] = (k[q] >> shift) & 0xF;
    } else {
      d[q] = -1;
    }
  }
  for (int b = 0; b < RS_BINS; b++) cnt[b * RS_THREADS + t] = 0;
  if (t < RS_BINS) tile_off[t] = hist[t * ntiles + blockIdx.x];
  __syncthreads();
  uint32_t local_rank[RS_ITEMS];
#pragma unroll
  for (int q = 0; q < RS_ITEMS; q++) {
    if (d[q] >= 0) {
      local_rank[q] = cnt[d[q] * RS_THREADS + t];
      cnt[d[q] * RS_THREADS + t] += 1;
    }
  }
  __syncthreads();
  // exclusive scan over cnt[0 .. 16*256) in digit-major order: each thread
  // owns 16 consecutive entries
  uint32_t mine[RS_BINS];
  uint32_t s = 0;
#pragma unroll
  for (int q = 0; q < RS_BINS; q++) {
    mine[q] = cnt[t * RS_BINS + q];
    s += mine[q];
  }
  // warp scan of s
  const int lane = t & 31, w = t >> 5;
  uint32_t x = s;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (t < 32) {
    uint32_t ws = (t < RS_THREADS / 32) ? wsum[t] : 0u;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, ws, off);
      if (t >= off) ws += y;
    }
    if (t < RS_THREADS / 32) wsum[t] = ws;
  }
  __syncthreads();
  uint32_t excl = x - s + (w > 0 ? wsum[w - 1] : 0u);
  __syncthreads();
#pragma unroll
  for (int q = 0; q < RS_BINS; q++) {
    cnt[t * RS_BINS + q] = excl;
    excl += mine[q];
  }
  __syncthreads();
  // digit start inside the tile = scanned value at [digit][thread 0]
#pragma unroll
  for (int q = 0; q < RS_ITEMS; q++) {
    if (d[q] >= 0) {
      uint32_t tile_digit_start = cnt[d[q] * RS_THREADS];
      uint32_t rank = cnt[d[q] * RS_THREADS + t] - tile_digit_start + local_rank[q];
      uint32_t pos = tile_off[d[q]] + rank;
      keys_out[pos] = k[q];
      vals_out[pos] = v[q];
    }
  }
}

__global__ void rs_iota(uint32_t* __restrict__ v, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (uint32_t)i;
}

struct RadixSorter {
  uint32_t* keys_alt = nullptr;
  uint32_t* vals_alt = nullptr;
  uint32_t* hist = nullptr;
  int cap = 0;

  cudaError_t reserve(int n) {
    if (n <= cap) return cudaSuccess;
    release();
    int ntiles = (n + RS_TILE - 1) / RS_TILE;
    cudaError_t e;
    if ((e = cudaMalloc(&keys_alt, sizeof(uint32_t) * (size_t)n))) return e;
    if ((e = cudaMalloc(&vals_alt, sizeof(uint32_t) * (size_t)n))) return e;
    if ((e = cudaMalloc(&hist, sizeof(uint32_t) * (size_t)RS_BINS * ntiles))) return e;
    cap = n;
    return cudaSuccess;
  }
  void release() {
    if (keys_alt) cudaFree(keys_alt);
    if (vals_alt) cudaFree(vals_alt);
    if (hist) cudaFree(hist);
    keys_alt = vals_alt = hist = nullptr;
    cap = 0;
  }
  // Sorts keys (values = 0..n-1 on input) in place; `bits` = key width.
  // Returns the number of kernel launches issued.
  int sort(uint32_t* keys, uint32_t* vals, int n, int bits, cudaStream_t st) {
    if (n <= 0) return 0;
    int ntiles = (n + RS_TILE - 1) / RS_TILE;
    int launches = 0;
    rs_iota<<<(n + 255) / 256, 256, 0, st>>>(vals, n);
    launches++;
    uint32_t *ka = keys, *va = vals, *kb = keys_alt, *vb = vals_alt;
    const int passes = (bits + 3) / 4;
    for (int p = 0; p < passes; p++) {
      int shift = 4 * p;
      rs_count<<<ntiles, RS_THREADS, 0, st>>>(ka, n, shift, hist, ntiles);
      rs_scan<<<1, 1024, 0, st>>>(hist, RS_BINS * ntiles);
      rs_scatter<<<ntiles, RS_THREADS, 0, st>>>(ka, va, kb, vb, n, shift, hist, ntiles);
      launches += 3;
      uint32_t* t;
      t = ka; ka = kb; kb = t;
      t = va; va = vb; vb = t;
    }
    if (ka != keys) {  // odd pass count: the result is in the spare buffers
      cudaMemcpyAsync(keys, ka, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(vals, va, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st);
    }
    return launches;
  }
};

}  // namespace plume
