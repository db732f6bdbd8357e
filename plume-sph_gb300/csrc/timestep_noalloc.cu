// timestep_noalloc.cu -- time-step reduction that allocates nothing.
//
// Some callers cannot allocate GPU memory when they need a time step: hosts
// whose device memory is owned by their own pool (a framework's caching
// allocator, an application that reserves all memory at start-up) and
// forbid allocations outside it, and code paths where an allocation would
// synchronise the device.  plume_timestep_noalloc computes the same value as
// the dt reduction inside plume_step -- CFL * min(h / c) over the particles
// that update their state (bc_type 100 or 99) -- from arrays the caller
// passes, with its scratch (one partial minimum per block) in a file-scope
// device array instead of memory it would allocate.
//
//   - The array holds PLUME_NOALLOC_MAX_BLOCKS doubles (8 KiB) on every GPU
//     that loads the library, until the process exits.  Each block covers
//     PLUME_NOALLOC_CHUNK particles, so n is limited to
//     PLUME_NOALLOC_MAX_BLOCKS * PLUME_NOALLOC_CHUNK (16,777,216); larger n is
//     rejected with PLUME_E_CAPACITY.
//   - Host code cannot use the array's name as a device address.  The first
//     call on each device looks the address up with cudaGetSymbolAddress
//     (with that device current) and caches it; make that first call on a
//     device before any stream capture.
//   - Every call reuses the same array.  A call writes every partial it
//     reads, so nothing has to be cleared between calls, but calls that
//     overlap on the GPU (for example on two streams) race on the array.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/plume_gpu.h"

namespace {

constexpr int THREADS = 256;
constexpr int ITEMS = PLUME_NOALLOC_CHUNK / THREADS;
constexpr int MAXDEV = 64;

static __device__ __align__(256) double g_dt_partial[PLUME_NOALLOC_MAX_BLOCKS];

std::mutex g_lock;
double* g_partial_addr[MAXDEV] = {};

__global__ void k_dt_partial(const double* __restrict__ h, const double* __restrict__ c,
                             const uint8_t* __restrict__ bc, size_t n, double* __restrict__ partial) {
  __shared__ double red[THREADS];
  const size_t base = (size_t)blockIdx.x * PLUME_NOALLOC_CHUNK;
  double m = 1.0e10;  // timestep.cc:99 starts from 1.0E+10
  bool bad = false;
  for (int k = 0; k < ITEMS; k++) {
    const size_t i = base + (size_t)k * THREADS + threadIdx.x;
    if (i < n && (bc[i] == 100 || bc[i] == 99)) {
      const double ci = c[i];
      if (!(ci > 0)) bad = true;
      const double t = h[i] / ci;
      if (t < m) m = t;
    }
  }
  red[threadIdx.x] = bad ? -1.0 : m;
  __syncthreads();
  for (int s = THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const double a = red[threadIdx.x], b = red[threadIdx.x + s];
      red[threadIdx.x] = (a < 0 || b < 0) ? -1.0 : fmin(a, b);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_dt_final(const double* __restrict__ partial, int nblocks, double cfl, double* __restrict__ dt_out) {
  __shared__ double red[1024];
  double m = 1.0e10;
  bool bad = false;
  for (int b = threadIdx.x; b < nblocks; b += 1024) {
    const double v = partial[b];
    if (v < 0) bad = true;
    m = fmin(m, v);
  }
  red[threadIdx.x] = bad ? -1.0 : m;
  __syncthreads();
  for (int s = 512; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const double a = red[threadIdx.x], b = red[threadIdx.x + s];
      red[threadIdx.x] = (a < 0 || b < 0) ? -1.0 : fmin(a, b);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *dt_out = (red[0] < 0) ? __longlong_as_double(0x7ff8000000000000ll) : cfl * red[0];
}

}  // namespace

extern "C" int plume_timestep_noalloc(const double* h, const double* c, const uint8_t* bc_type, size_t n,
                                      double cfl, double* dt_out, void* stream) {
  if (!h || !c || !bc_type || !dt_out) return PLUME_E_INVALID;
  if (n > (size_t)PLUME_NOALLOC_MAX_BLOCKS * PLUME_NOALLOC_CHUNK) return PLUME_E_CAPACITY;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAXDEV) return PLUME_E_CUDA;
  double* partial = nullptr;
  {
    std::lock_guard<std::mutex> g(g_lock);
    if (!g_partial_addr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_dt_partial) != cudaSuccess || !p) return PLUME_E_CUDA;
      g_partial_addr[dev] = static_cast<double*>(p);
    }
    partial = g_partial_addr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nb = n ? (int)((n + PLUME_NOALLOC_CHUNK - 1) / PLUME_NOALLOC_CHUNK) : 0;
  if (nb > 0) k_dt_partial<<<nb, THREADS, 0, st>>>(h, c, bc_type, n, partial);
  k_dt_final<<<1, 1024, 0, st>>>(partial, nb, cfl, dt_out);
  return cudaGetLastError() == cudaSuccess ? PLUME_OK : PLUME_E_CUDA;
}
