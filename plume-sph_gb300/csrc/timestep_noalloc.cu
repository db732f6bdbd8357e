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
//     (with that device current) and caches it together with the unique id
//     of the device's current context; a later call in another context of
//     that device (after cudaDeviceReset, say) looks it up again.  Make the
//     first call on a device before any stream capture.
//   - Every call reuses the same array.  A call writes every partial it
//     reads, so nothing has to be cleared between calls, but calls that
//     overlap on the GPU (for example on two streams) race on the array.
//   - A particle with h <= 0, c <= 0 or either NaN (among bc_type 100/99)
//     makes the result NaN; the flag travels beside the minimum, so no
//     valid minimum is mistaken for it.
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
unsigned long long g_partial_ctx[MAXDEV] = {};  // unique id of the context the address belongs to

// cuCtxGetId (driver API, CUDA >= 12.0) through the runtime's entry-point
// query, so the library needs no link against the driver library: the
// unique id of the current context, or false when there is none or the
// driver lacks the call
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);
bool current_ctx_id(unsigned long long* id) {
  static CtxGetIdFn fn = nullptr;
  static bool looked = false;
  if (!looked) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetIdFn>(p);
    looked = true;
  }
  return fn && fn(nullptr, id) == 0;
}

// NaN: the "bad particle" value of a partial (never a minimum of h / c > 0)
__device__ __forceinline__ double bad_value() { return __longlong_as_double(0x7ff8000000000000ll); }

__global__ void k_dt_partial(const double* __restrict__ h, const double* __restrict__ c,
                             const uint8_t* __restrict__ bc, size_t n, double* __restrict__ partial) {
  __shared__ double red[THREADS];
  const size_t base = (size_t)blockIdx.x * PLUME_NOALLOC_CHUNK;
  double m = 1.0e10;  // timestep.cc:99 starts from 1.0E+10
  int bad = 0;
  for (int k = 0; k < ITEMS; k++) {
    const size_t i = base + (size_t)k * THREADS + threadIdx.x;
    if (i < n && (bc[i] == 100 || bc[i] == 99)) {
      const double ci = c[i];
      const double t = h[i] / ci;
      if (!(ci > 0) || !(t > 0)) bad = 1;
      else if (t < m) m = t;
    }
  }
  red[threadIdx.x] = m;
  bad = __syncthreads_or(bad);
  for (int s = THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmin(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = bad ? bad_value() : red[0];
}

__global__ void k_dt_final(const double* __restrict__ partial, int nblocks, double cfl, double* __restrict__ dt_out) {
  __shared__ double red[1024];
  double m = 1.0e10;
  int bad = 0;
  for (int b = threadIdx.x; b < nblocks; b += 1024) {
    const double v = partial[b];
    if (v != v) bad = 1;
    else m = fmin(m, v);
  }
  red[threadIdx.x] = m;
  bad = __syncthreads_or(bad);
  for (int s = 512; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmin(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *dt_out = bad ? bad_value() : cfl * red[0];
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
    unsigned long long id = 0;
    const bool have_id = current_ctx_id(&id);
    if (!g_partial_addr[dev] || (have_id && id != g_partial_ctx[dev])) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_dt_partial) != cudaSuccess || !p) return PLUME_E_CUDA;
      g_partial_addr[dev] = static_cast<double*>(p);
      // the lookup made the device's primary context current if none was
      unsigned long long id2 = 0;
      g_partial_ctx[dev] = current_ctx_id(&id2) ? id2 : 0ull;
    }
    partial = g_partial_addr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nb = n ? (int)((n + PLUME_NOALLOC_CHUNK - 1) / PLUME_NOALLOC_CHUNK) : 0;
  if (nb > 0) k_dt_partial<<<nb, THREADS, 0, st>>>(h, c, bc_type, n, partial);
  k_dt_final<<<1, 1024, 0, st>>>(partial, nb, cfl, dt_out);
  return cudaGetLastError() == cudaSuccess ? PLUME_OK : PLUME_E_CUDA;
}
