// plume_gpu.cu -- context, step orchestration and the C ABI of
// include/plume_gpu.h.
//
// One step (src/plume/main.cc:217-471 in 3D, :676-750 in 1D):
//   k_dt_reduce + k_incrtime      timestep (timestep.cc:94-183) and
//                                 TimeProps::incrtime (properties.h:71-83)
//   search                        cell keys, radix sort, gather, cell_start
//                                 (replaces search_neighs_consth and the
//                                 bucket lists of update_particles_in_bucket)
//   k_adaptive                    adaptive_sml every sml_interval steps
//   k_momentum + k_commit_mom     mom_engr_update
//   k_density + k_commit_dens     smooth_density
//   k_velocity                    smooth_velocity (LANS)
//   k_update_pos                  update_pos + deletions of the re-bucketing
//   k_end_step                    TimeProps::ifoutput (properties.h:100-118)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <climits>

#include "../../include/plume_gpu.h"
#include "radix_sort.cuh"
#include "sph_kernels.cuh"
#include "sph_warp.cuh"
#include "sph_gsph.cuh"
#include "sph_adjoint.cuh"

using namespace plume;

namespace {

constexpr int NTHREADS = 128;
static_assert(NTHREADS == 32 * WP_WARPS, "warp kernels: 4 warps per block");
// phases of plume_phase_times: 0 search, 1 adaptive, 2 hmax + lists, 3 momentum,
// 4 commit_mom, 5 density, 6 commit_dens, 7 velocity, 8 position, 9 dt,
// 10 total, 11 the momentum pair-sweep kernel alone (part of 3), 12 inlet +
// step end, 13 wall boundary
constexpr int NPHASE = 14;
constexpr int NEV = 14;

inline int nblocks(size_t n, int t = NTHREADS) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ unsigned long long dbits(double v) { return (unsigned long long)__double_as_longlong(v); }

// ---- dt: min over need_neigh of h/c (timestep.cc:94-135), per member ----
// A block whose particles belong to one member (the common case: particles
// are sorted by member) reduces in shared memory and issues one atomic per
// quantity; a block that straddles members falls back to per-particle atomics.
__global__ void k_dt_reduce(Dev A, const int* __restrict__ d_count, TimeState* ts_all) {
  __shared__ double red[NTHREADS];
  __shared__ unsigned int nr[NTHREADS];
  __shared__ int bm, straddle;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 1.0e10;
  unsigned int real = 0;
  int m = -1;
  if (threadIdx.x == 0) { bm = -1; straddle = 0; }
  __syncthreads();
  if (i < *d_count && need_neigh(A.bc[i])) {
    m = A.mem[i];
    TimeState* ts = ts_all + m;
    if (ts->active) {
      double c = A.c[i];
      if (!(c > 0)) set_status(ts, 4);
      double t = A.h[i] / c;
      if (t < v) v = t;
      real = 1;
      atomicCAS(&bm, -1, m);
    } else {
      m = -1;
    }
  }
  __syncthreads();
  if (m >= 0 && m != bm) straddle = 1;
  __syncthreads();
  if (straddle) {
    if (m >= 0) {
      if (v > 0 && v == v) atomicMin(&ts_all[m].dtmin_bits, dbits(v));
      atomicAdd(&ts_all[m].n_real, 1ull);
    }
    return;
  }
  red[threadIdx.x] = v;
  nr[threadIdx.x] = real;
  __syncthreads();
  for (int s = NTHREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      red[threadIdx.x] = fmin(red[threadIdx.x], red[threadIdx.x + s]);
      nr[threadIdx.x] += nr[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && bm >= 0) {
    double mn = red[0];
    if (mn > 0 && mn == mn) atomicMin(&ts_all[bm].dtmin_bits, dbits(mn));
    if (nr[0]) atomicAdd(&ts_all[bm].n_real, (unsigned long long)nr[0]);
  }
}

// TimeProps::incrtime and iferupt, one thread per member
__global__ void k_incrtime(const Opt* __restrict__ mopt, TimeState* ts_all, int nmem) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmem) return;
  TimeState* ts = ts_all + m;
  if (!ts->active) return;
  const Opt& o = mopt[m];
  double dt = o.cfl * __longlong_as_double((long long)ts->dtmin_bits);
  if ((ts->time + dt) > ts->ndtimeoutput) dt = ts->ndtimeoutput - ts->time;
  if ((ts->time + dt) > o.max_time) dt = o.max_time - ts->time;
  ts->time += dt;
  ts->dtime = dt;
  ts->step++;
  ts->erupt = !((ts->time * 1.0) < o.stat_erupt) && !((ts->time * 1.0) > o.end_erupt);
}

// TimeProps::ifoutput
__global__ void k_end_step(const Opt* __restrict__ mopt, TimeState* ts_all, int nmem) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmem) return;
  TimeState* ts = ts_all + m;
  if (!ts->active) return;
  const Opt& o = mopt[m];
  if (ts->time >= ts->ndtimeoutput || ts->time == o.max_time) {
    ts->ioutput++;
    ts->ndtimeoutput = ((ts->ioutput + 1) * o.timeoutput) / 1.0;
  }
}
// start of a step: which members step (a frozen member stops at
// TimeProps::ifend, properties.h:76-79, or at its first error status, where
// the reference asserts), reset of the per-step reductions, and the
// context's step counter (adaptive_sml schedule)
__global__ void k_begin_step(const Opt* __restrict__ mopt, TimeState* ts_all, int nmem, int* hstep) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m == 0) (*hstep)++;
  if (m >= nmem) return;
  TimeState* ts = ts_all + m;
  const Opt& o = mopt[m];
  ts->active = !(ts->freeze && ((ts->time >= o.max_time) || (ts->step > o.max_steps) || ts->status != 0));
  ts->dtmin_bits = dbits(1.0e10);
  ts->n_real = 0;
}

// ---- search --------------------------------------------------------------
// key = the member's cell base + the fine cell inside the member's grid, so
// that the sort groups particles by member, then by cell
__global__ void k_keys(const Geo* __restrict__ geo, Dev A, int n, uint32_t* __restrict__ keys, uint32_t ncells,
                       TimeState* ts_all) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (A.bc[i] == BC_DEAD) {
    keys[i] = ncells;
    return;
  }
  const int m = A.mem[i];
  TimeState* ts = ts_all + m;
  const Geo g = geo[m];
  bool o1 = false, o2 = false, o3 = false;
  int b0, b1 = 0, b2 = 0;
  int c0 = cell_axis(g, 0, A.x[i], &b0, &o1);
  int c1 = 0, c2 = 0;
  if (g.dim == 3) {
    c1 = cell_axis(g, 1, A.y[i], &b1, &o2);
    c2 = cell_axis(g, 2, A.z[i], &b2, &o3);
  }
  if (o1 || o2 || o3) {
    set_status(ts, 6);
    keys[i] = ncells;
    A.bc[i] = BC_DEAD;
    return;
  }
  keys[i] = g.cell_base + (uint32_t)(((size_t)c2 * g.G[1] + c1) * g.G[0] + c0);
  A.bkt[i] = (g.dim == 3) ? (b2 * g.nb[1] + b1) * g.nb[0] + b0 : b0;
}

__global__ void k_gather(const Geo* __restrict__ geo, Dev A, Dev B, Work W, const uint32_t* __restrict__ perm,
                         int n) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int q = perm[p];
  const int m = A.mem[q];
  const Geo g = geo[m];
  B.mem[p] = (uint16_t)m;
  B.key[p] = A.key[q];
  B.x[p] = A.x[q];
  B.vx[p] = A.vx[q];
  B.vsx[p] = A.vsx[q];
  if (g.dim == 3) {
    B.y[p] = A.y[q]; B.z[p] = A.z[q];
    B.vy[p] = A.vy[q]; B.vz[p] = A.vz[q];
    B.vsy[p] = A.vsy[q]; B.vsz[p] = A.vsz[q];
  }
  B.mass[p] = A.mass[q];
  double h = A.h[q];
  B.h[p] = h;
  W.hlist[p] = h;
  B.rho[p] = A.rho[q];
  B.e[p] = A.e[q];
  B.p[p] = A.p[q];
  B.Y[p] = A.Y[q];
  B.gam[p] = A.gam[q];
  B.c[p] = A.c[q];
  B.T[p] = A.T[q];
  B.cp[p] = A.cp[q];
  B.phase[p] = A.phase[q];
  B.bc[p] = A.bc[q];
  B.inv[p] = A.inv[q];
  int b = A.bkt[q];
  B.bkt[p] = b;
  {  // bucket-relative coordinates serve both paths (cell ranges)
    int bi[3];
    if (g.dim == 3) {
      bi[0] = b % g.nb[0];
      bi[1] = (b / g.nb[0]) % g.nb[1];
      bi[2] = b / (g.nb[0] * g.nb[1]);
      W.xr[p] = f32_rz(A.x[q] - (g.mind[0] + bi[0] * g.del));
      W.yr[p] = f32_rz(A.y[q] - (g.mind[1] + bi[1] * g.del));
      W.zr[p] = f32_rz(A.z[q] - (g.mind[2] + bi[2] * g.del));
    } else {
      W.xr[p] = f32_rz(A.x[q] - (g.mind[0] + b * g.del));
    }
  }
}

// cell_start[c] = first sorted index with key >= c, c in [0, ncells + 1]:
// one thread per cell, binary search over the sorted keys (long runs of
// empty cells above and below the particles cost nothing extra)
__global__ void k_cell_start(const uint32_t* __restrict__ skeys, int n, uint32_t ncells,
                             uint32_t* __restrict__ cs, int* d_count) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c > (long long)ncells + 1) return;
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if ((long long)skeys[mid] < c) lo = mid + 1; else hi = mid;
  }
  cs[c] = (uint32_t)lo;
  if (c == (long long)ncells) *d_count = lo;
}

__global__ void k_fill_cs(uint32_t* cs, uint32_t ncells, int* d_count) {
  size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c <= ncells + 1) cs[c] = 0;
  if (c == 0) *d_count = 0;
}

// ---- per-bucket maximum h (search radius of the h_ij sweeps) ------------
__global__ void k_hmax_reset(unsigned long long* hb, int nbk) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nbk) hb[b] = 0ull;
}
// per-bucket tables cover the buckets of every member (a 1D member has one
// entry: the maximum over all its particles)
// Per-bucket maximum h (1D: per member).  Positive doubles order like their
// bit patterns, so the maximum is an integer atomicMax.  In the sorted order
// a warp's particles mostly share one bucket (in 1D one member): such a warp
// reduces by shuffles and makes one atomic, where 32 atomics on one address
// would serialise; mixed warps fall back to one atomic per particle.
__global__ void k_hmax(const Geo* __restrict__ geo, Dev A, const int* __restrict__ d_count,
                       unsigned long long* hb, int dim) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool ok = i < *d_count && A.bc[i] != BC_DEAD;
  unsigned long long v = 0ull;
  int key = -1;
  if (ok) {
    v = dbits(A.h[i]);
    key = geo[A.mem[i]].bucket_base + (dim == 3 ? A.bkt[i] : 0);
  }
  const unsigned peers = __match_any_sync(0xffffffffu, key);
  if (peers == 0xffffffffu) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
      v = w > v ? w : v;
    }
    if ((threadIdx.x & 31) == 0 && key >= 0) atomicMax(&hb[key], v);
  } else if (ok) {
    atomicMax(&hb[key], v);
  }
}
__global__ void k_hmax27(const Geo* __restrict__ geo, const uint16_t* __restrict__ bmember, int nbk_all,
                         const unsigned long long* __restrict__ hb_all, double* __restrict__ h27_all) {
  int ba = blockIdx.x * blockDim.x + threadIdx.x;
  if (ba >= nbk_all) return;
  const Geo& g = geo[bmember[ba]];
  const unsigned long long* hb = hb_all + g.bucket_base;
  const int b = ba - g.bucket_base;
  if (g.dim != 3) {
    h27_all[ba] = __longlong_as_double((long long)hb[0]);
    return;
  }
  double* h27 = h27_all + g.bucket_base;
  int bx = b % g.nb[0], by = (b / g.nb[0]) % g.nb[1], bz = b / (g.nb[0] * g.nb[1]);
  double m = 0;
  for (int dz = -1; dz <= 1; dz++)
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) {
        int x = bx + dx, y = by + dy, z = bz + dz;
        if (x < 0 || y < 0 || z < 0 || x >= g.nb[0] || y >= g.nb[1] || z >= g.nb[2]) continue;
        m = fmax(m, __longlong_as_double((long long)hb[(z * g.nb[1] + y) * g.nb[0] + x]));
      }
  h27[b] = m;
}

// ---- neighbour pairs (plume_neighbor_pairs) -------------------------------
template <int D>
__global__ void k_pairs(int mode, Opt o, const Geo* __restrict__ geo, Dev A, Work W,
                        const uint32_t* __restrict__ cs_all, const int* __restrict__ d_count,
                        const unsigned long long* __restrict__ offs, unsigned int* __restrict__ cnt,
                        uint64_t* __restrict__ ki, uint64_t* __restrict__ kj,
                        const uint64_t* __restrict__ sub, int nsub) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int n = *d_count;
  if (i >= n) return;
  bool want = need_neigh(A.bc[i]);
  if (want && sub) {  // only the particles whose keys are in the sorted subset
    const uint64_t k = A.key[i];
    int lo = 0, hi = nsub;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (sub[mid] < k) lo = mid + 1; else hi = mid;
    }
    want = lo < nsub && sub[lo] == k;
  }
  if (!want) {
    if (!offs) cnt[i] = 0;
    return;
  }
  const Geo g = geo[A.mem[i]];
  const uint32_t* cs = cs_all + g.cell_base;
  double xi[3] = {A.x[i], D == 3 ? A.y[i] : 0.0, D == 3 ? A.z[i] : 0.0};
  int bi[3];
  bucket_coords<D>(g, A.bkt[i], bi);
  const double hi = A.h[i];
  const double Lb = o.list_factor * W.hlist[i];
  unsigned long long base = offs ? offs[i] : 0ull;
  unsigned int c = 0;
  auto take = [&](uint32_t j) {
    if (offs) {
      ki[base + c] = A.key[i];
      kj[base + c] = A.key[j];
    }
    c++;
  };
  if (mode == 0 && D == 1) {  // all particles of the member (add_air.cc:470-479)
    for (uint32_t j = cs[0]; j < cs[g.G[0]]; j++)
      if (A.bc[j] != BC_DEAD) take(j);
  } else {
    double R = (mode == 0) ? fmax(Lb, g.del) * (1.0 + 1e-10) : o.cutoff2 * hi * (1.0 + 1e-10);
    for_segments<D, double>(g, cs, xi, bi, R, [&](uint32_t j0, uint32_t j1, bool own, double, double, double) {
      for (uint32_t j = j0; j < j1; j++) {
        double xj[3] = {A.x[j], D == 3 ? A.y[j] : 0.0, D == 3 ? A.z[j] : 0.0};
        double dx[3];
        for (int k = 0; k < D; k++) dx[k] = xi[k] - xj[k];
        bool inlist = own || in_box<D, double>(dx, Lb);
        if (!inlist) continue;
        if (mode == 1) {
          if (j == (uint32_t)i) continue;
          if (!in_box<D, double>(dx, o.cutoff2 * hi)) continue;
          double h = 0.5 * (hi + A.h[j]);
          double si[3];
          for (int k = 0; k < D; k++) si[k] = dx[k] / h;
          if (kw<D, double>(o.kernel, si, h) == 0.0) continue;
        }
        take(j);
      }
    });
  }
  if (!offs) cnt[i] = c;
}

// exclusive scan of uint32 counts into uint64 offsets (three kernels)
__global__ void k_scan_blocks(const unsigned int* __restrict__ cnt, int n, unsigned long long* __restrict__ out,
                              unsigned long long* __restrict__ sums) {
  __shared__ unsigned long long s[1024];
  int t = threadIdx.x;
  int i = blockIdx.x * 1024 + t;
  s[t] = (i < n) ? cnt[i] : 0ull;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    unsigned long long v = (t >= off) ? s[t - off] : 0ull;
    __syncthreads();
    s[t] += v;
    __syncthreads();
  }
  if (i < n) out[i] = s[t] - cnt[i];
  if (t == 1023) sums[blockIdx.x] = s[t];
}
// exclusive scan of the m block sums by one CTA of 1024 threads
__global__ void k_scan_sums(unsigned long long* sums, int m, unsigned long long* total) {
  __shared__ unsigned long long part[1024];
  const int t = threadIdx.x;
  const int per = (m + 1023) / 1024;
  const int lo = t * per, hi = min(lo + per, m);
  unsigned long long s = 0;
  for (int b = lo; b < hi; b++) s += sums[b];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    unsigned long long v = (t >= off) ? part[t - off] : 0ull;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  unsigned long long run = (t == 0) ? 0ull : part[t - 1];
  for (int b = lo; b < hi; b++) {
    unsigned long long v = sums[b];
    sums[b] = run;
    run += v;
  }
  if (t == 1023) *total = part[1023];
}
__global__ void k_scan_add(unsigned long long* out, int n, const unsigned long long* __restrict__ sums) {
  int i = blockIdx.x * 1024 + threadIdx.x;
  if (i < n) out[i] += sums[blockIdx.x];
}

// ---- ghost state (plume_set_ghost_state) -----------------------------------
__global__ void k_set_ghost(const Opt* __restrict__ mopt, Dev A, const int* __restrict__ d_count,
                            const uint64_t* __restrict__ keys, const double* __restrict__ state,
                            const double* __restrict__ Yin, int m, int dim) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count) return;
  const Opt& o = mopt[A.mem[i]];
  uint64_t k = A.key[i];
  int lo = 0, hi = m;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (keys[mid] < k) lo = mid + 1; else hi = mid;
  }
  if (lo >= m || keys[lo] != k) return;
  const int w = dim + 2;
  const double* s = state + (size_t)lo * w;
  A.rho[i] = s[0];
  A.vx[i] = s[1];
  if (dim == 3) { A.vy[i] = s[2]; A.vz[i] = s[3]; }
  A.e[i] = s[w - 1];
  if (Yin) A.Y[i] = Yin[lo];
  double gam, p, c, T, cp = A.cp[i];
  eos(o, A.rho[i], A.Y[i], A.e[i], gam, p, c, T, cp, o.lans != 0);
  A.gam[i] = gam; A.p[i] = p; A.c[i] = c; A.T[i] = T; A.cp[i] = cp;
}

// ---- wall boundary (apply_bcond, bcond.cc:24-249, BC_FOR_KX 1) ------------
// Maps every live wall ghost (bc 2) to its image by key (binary search of
// the key-sorted image table): map[member * nimg + image] = row.  A ghost
// without an image is left alone, as in the reference.
__global__ void k_bc_map(Dev A, const int* __restrict__ d_count, const uint64_t* __restrict__ ikey, int nimg,
                         int* __restrict__ map) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count || A.bc[i] != 2) return;
  const uint64_t k = A.key[i];
  int l = 0, h = nimg;
  while (l < h) {
    const int mid = (l + h) >> 1;
    if (ikey[mid] < k) l = mid + 1; else h = mid;
  }
  if (l < nimg && ikey[l] == k) map[(size_t)A.mem[i] * nimg + l] = i;
}

// BCG threads per (member, image) slot, slots in image-key order, so that
// the threads of a warp walk overlapping candidate sets together: the
// Shepard-normalised SPH averages of rho, v, e of the real and
// pressure-ghost particles (contr_image, particle.h:562-565) inside CUTOFF2
// h_j of the image point, over the image's bucket and its 26 neighbours (Y
// over the neighbours only, as the reference accumulates it); the velocity
// reflected in the wall along the ghost-to-image direction (reflect,
// sph_lib.cc:76-83), written to the ghost with its EOS.  Runs after the
// step's sort, where the reference runs it at the end of the previous step
// (main.cc:196, 468): nothing in between reads ghost states.
// The walk goes over rows of fine cells, dealt round-robin to the slot's
// threads (partial sums combined by shuffles): the x-run of a row is
// contiguous in the sorted order across bucket boundaries, so one loop takes
// the whole run and finds a candidate's bucket (at most three along x) from
// the two boundary rows.  T = double: the reference's FP64 arithmetic on absolute
// coordinates; T = float (mixed path): FP32 weights on bucket-relative
// coordinates, fields narrowed on the integer pipe, compensated FP32 sums.
constexpr int BCG = 8;  // threads per image slot (a power of two dividing 32)

// wall-boundary candidate records of the mixed path, written after the
// step's sort: P (xr, yr, zr, h; -h when the particle is not a real or
// pressure-ghost particle, contr_image), Q (m, m/rho, e, Y), R (vx, vy, vz)
__global__ void k_pack_bc(Dev A, Packed K, Work W, const int* __restrict__ d_count) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= *d_count) return;
  const uint8_t bc = A.bc[j];
  const bool c = bc == 100 || bc == 99 || bc == 1;
  const float h = f32_rz(A.h[j]);
  const float m = f32_rz(A.mass[j]);
  K.P[j] = make_float4(W.xr[j], W.yr[j], W.zr[j], c ? h : -h);
  K.Q[j] = make_float4(m, m * __fdividef(1.0f, f32_rz(A.rho[j])), f32_rz(A.e[j]), f32_rz(A.Y[j]));
  K.R[j] = make_float4(f32_rz(A.vx[j]), f32_rz(A.vy[j]), f32_rz(A.vz[j]), 0.0f);
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS) k_apply_bcond(const Opt* __restrict__ mopt, const Geo* __restrict__ geo,
                                                          Dev A, Work W, Packed K, const uint32_t* __restrict__ cs_all,
                                                          const double* __restrict__ h27_all,
                                                          const int* __restrict__ map, int nslots, int nimg,
                                                          const double* __restrict__ ixyz, TimeState* ts_all) {
  constexpr bool MIXED = sizeof(T) == 4;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = gt / BCG, sub = gt % BCG;
  if (t >= nslots) return;
  // the slot's threads are BCG consecutive lanes; they leave together
  const unsigned gmask = ((1u << BCG) - 1u) << ((threadIdx.x & 31) & ~(BCG - 1));
  const int i = map[t];
  if (i < 0) return;
  const int lo = t % nimg;
  const int m = A.mem[i];
  const Geo& g = geo[m];
  const Opt& o = mopt[m];
  TimeState* ts = ts_all + m;
  const uint32_t* cs = cs_all + g.cell_base;
  const double refc[3] = {ixyz[3 * lo], ixyz[3 * lo + 1], ixyz[3 * lo + 2]};
  bool o1, o2, o3;
  int bi[3];
  bi[0] = bucket_axis(refc[0], g.mind[0], g.del, g.idel, g.nb[0], &o1);
  bi[1] = bucket_axis(refc[1], g.mind[1], g.del, g.idel, g.nb[1], &o2);
  bi[2] = bucket_axis(refc[2], g.mind[2], g.del, g.idel, g.nb[2], &o3);
  if (o1 || o2 || o3) {
    if (!sub) set_status(ts, 6);
    return;
  }
  const int b = (bi[2] * g.nb[1] + bi[1]) * g.nb[0] + bi[0];
  const double R = o.ksupport * h27_all[g.bucket_base + b] * (1.0 + 1e-10);
  // the image point relative to its bucket (mixed path)
  const float ir[3] = {(float)(refc[0] - (g.mind[0] + bi[0] * g.del)),
                       (float)(refc[1] - (g.mind[1] + bi[1] * g.del)),
                       (float)(refc[2] - (g.mind[2] + bi[2] * g.del))};
  // cell box of the walk: the reach R, clipped to the 27 buckets (the mixed
  // path takes the conservative FP32 range; the weights test exactly)
  int clo[3], chi[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if constexpr (MIXED) {
      cell_range(g, a, bi[a], ir[a], R, clo[a], chi[a]);
    } else {
      const int l = cell_axis(g, a, refc[a] - R, nullptr, nullptr);
      const int h = cell_axis(g, a, refc[a] + R, nullptr, nullptr);
      clo[a] = max(l, max((bi[a] - 1) * g.s, 0));
      chi[a] = min(h, min((bi[a] + 2) * g.s - 1, g.G[a] - 1));
    }
  }
  const float delf = (float)g.del;
  const float c2f = (float)o.cutoff2;
  Acc<T> a0, a1, a2, a3, a4, aw, ak;
  const int bx0 = clo[0] / g.s;  // bucket of the first cell of every x-run
  const int ny = chi[1] - clo[1] + 1, nrow = ny * (chi[2] - clo[2] + 1);
  for (int r = sub; r < nrow; r += BCG) {
    const int cz = clo[2] + r / ny, cy = clo[1] + r % ny;
    const int bz = cz / g.s;
    {
      const int by = cy / g.s;
      const size_t rowbase = ((size_t)cz * g.G[1] + cy) * (size_t)g.G[0];
      const uint32_t j0 = cs[rowbase + clo[0]], j1 = cs[rowbase + chi[0] + 1];
      const int c1 = (bx0 + 1) * g.s, c2 = (bx0 + 2) * g.s;
      const uint32_t s1 = c1 <= chi[0] ? cs[rowbase + c1] : j1;
      const uint32_t s2 = c2 <= chi[0] ? cs[rowbase + c2] : j1;
      const int own_run = (by == bi[1] && bz == bi[2]) ? bi[0] - bx0 : -1;
      const float oy = (float)(bi[1] - by) * delf, oz = (float)(bi[2] - bz) * delf;
      const float ox0 = (float)(bi[0] - bx0) * delf;
      for (uint32_t j = j0; j < j1; j++) {
        const int run = (j >= s1) + (j >= s2);
        const bool own = run == own_run;
        if constexpr (MIXED) {
          // packed records (k_pack_bc); the field records are read only
          // inside the kernel's support (zero weight outside)
          const float4 p = K.P[j];
          if (!(p.w > 0.0f)) continue;
          const float ox = ox0 - (float)run * delf;
          const float ds[3] = {ir[0] + ox - p.x, ir[1] + oy - p.y, ir[2] + oz - p.z};
          if (!in_box<3, float>(ds, c2f * p.w)) continue;
          const float ih = __fdividef(1.0f, p.w);
          const float sv[3] = {ds[0] * ih, ds[1] * ih, ds[2] * ih};
          if (fabsf(sv[0]) > 3.0f || fabsf(sv[1]) > 3.0f || fabsf(sv[2]) > 3.0f) continue;
          const float4 q = K.Q[j], rv = K.R[j];
          const float rn = float(T1_INV_SQRT_PI) * ih;
          const float w = rn * rn * rn * __expf(-(sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2]));
          const float mw = q.x * w;
          const float mwr = q.y * w;
          a0.add(mw);
          a1.add(mwr * rv.x);
          a2.add(mwr * rv.y);
          a3.add(mwr * rv.z);
          a4.add(mwr * q.z);
          if (!own) ak.add(mwr * q.w);
          aw.add(mwr);
        } else {
          const uint8_t bc = A.bc[j];
          if (!(bc == 100 || bc == 99 || bc == 1)) continue;
          const double h = A.h[j];
          const double ds[3] = {refc[0] - A.x[j], refc[1] - A.y[j], refc[2] - A.z[j]};
          if (!in_box<3, double>(ds, o.cutoff2 * h)) continue;
          const double sv[3] = {ds[0] / h, ds[1] / h, ds[2] / h};
          // zero weight beyond |s_k| = 3 (w_gauss): adds nothing
          if (fabs(sv[0]) > KCUTOFF || fabs(sv[1]) > KCUTOFF || fabs(sv[2]) > KCUTOFF) continue;
          const double w = w_gauss<3, double>(sv, h);
          const double mj = A.mass[j], rj = A.rho[j];
          a0.add(mj * w);
          a1.add(mj * w * A.vx[j] / rj);
          a2.add(mj * w * A.vy[j] / rj);
          a3.add(mj * w * A.vz[j] / rj);
          a4.add(mj * w * A.e[j] / rj);
          if (!own) ak.add(mj * w * A.Y[j] / rj);
          aw.add(mj * w / rj);
        }
      }
    }
  }
  // the slot's partial sums: FP32 on the mixed path (eight terms), FP64 else
  T q0 = a0.get(), q1 = a1.get(), q2 = a2.get(), q3 = a3.get(), q4 = a4.get(), qw = aw.get(), qk = ak.get();
#pragma unroll
  for (int off = BCG / 2; off > 0; off >>= 1) {
    q0 += __shfl_xor_sync(gmask, q0, off);
    q1 += __shfl_xor_sync(gmask, q1, off);
    q2 += __shfl_xor_sync(gmask, q2, off);
    q3 += __shfl_xor_sync(gmask, q3, off);
    q4 += __shfl_xor_sync(gmask, q4, off);
    qw += __shfl_xor_sync(gmask, qw, off);
    qk += __shfl_xor_sync(gmask, qk, off);
  }
  if (sub) return;
  double u0 = q0, u1 = q1, u2 = q2, u3 = q3, u4 = q4, wn = qw, ks = qk;
  if (wn > 0.) {
    u0 /= wn; u1 /= wn; u2 /= wn; u3 /= wn; u4 /= wn;
    ks = ks / wn;
  } else {
    u0 = 1.; u1 = u2 = u3 = u4 = 0.;
    ks = 0.0;
  }
  double normal[3] = {refc[0] - A.x[i], refc[1] - A.y[i], refc[2] - A.z[i]};
  const double d = sqrt(normal[0] * normal[0] + normal[1] * normal[1] + normal[2] * normal[2]);
#pragma unroll
  for (int a = 0; a < 3; a++) normal[a] /= d;
  const double vdotn = u1 * normal[0] + u2 * normal[1] + u3 * normal[2];
  A.rho[i] = u0;
  A.vx[i] = u1 - 2 * vdotn * normal[0];
  A.vy[i] = u2 - 2 * vdotn * normal[1];
  A.vz[i] = u3 - 2 * vdotn * normal[2];
  A.e[i] = u4;
  A.Y[i] = ks;
  double gam, p, c, temp, cp = A.cp[i];
  eos(o, u0, ks, u4, gam, p, c, temp, cp, o.lans != 0);
  A.gam[i] = gam; A.p[i] = p; A.c[i] = c; A.T[i] = temp; A.cp[i] = cp;
}

// ---- domain growth (scan_outside_layer.cc:37-121, adapt_domain.cc:41-194)
// Bucket types as the flags give them: explicit UNDERGROUND / PRESS_BC, else
// an absorbing bucket is below (both z faces -1) or beside the ground.
__device__ __forceinline__ int btype_of(uint8_t f, const int8_t* fi, bool explicit_types) {
  if (f & PLUME_BUCKET_MIXED) return 3;
  if (f & PLUME_BUCKET_UNDERGROUND) return 1;
  if (f & PLUME_BUCKET_PRESS_BC) return 2;
  if ((f & PLUME_BUCKET_ABSORBING) && !explicit_types) return (fi && fi[4] == -1 && fi[5] == -1) ? 1 : 2;
  return 4;  // OVERGROUND
}

// particles of member-local bucket b: its s x s rows of s fine cells
template <class F>
__device__ __forceinline__ void for_bucket_rows(const Geo& g, const uint32_t* __restrict__ cs, int b, F&& f) {
  const int bx = b % g.nb[0], by = (b / g.nb[0]) % g.nb[1], bz = b / (g.nb[0] * g.nb[1]);
  for (int cz = bz * g.s; cz < bz * g.s + g.s; cz++)
    for (int cy = by * g.s; cy < by * g.s + g.s; cy++) {
      const size_t row = ((size_t)cz * g.G[1] + cy) * (size_t)g.G[0] + (size_t)bx * g.s;
      f(cs[row], cs[row + g.s]);
    }
}

__device__ __forceinline__ uint32_t bucket_count(const Geo& g, const uint32_t* __restrict__ cs, int b) {
  uint32_t c = 0;
  for_bucket_rows(g, cs, b, [&](uint32_t j0, uint32_t j1) { c += j1 - j0; });
  return c;
}

// calls f(neighbour bucket) for the in-grid neighbours of b until f is true
template <class F>
__device__ __forceinline__ bool any_neighbour(const Geo& g, int b, F&& f) {
  const int bx = b % g.nb[0], by = (b / g.nb[0]) % g.nb[1], bz = b / (g.nb[0] * g.nb[1]);
  for (int dz = -1; dz <= 1; dz++)
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) {
        if (!dx && !dy && !dz) continue;
        const int cx = bx + dx, cy = by + dy, cz = bz + dz;
        if (cx < 0 || cx >= g.nb[0] || cy < 0 || cy >= g.nb[1] || cz < 0 || cz >= g.nb[2]) continue;
        if (f((cz * g.nb[1] + cy) * g.nb[0] + cx)) return true;
      }
  return false;
}

// One thread per bucket: a POTENTIAL bucket holding an involved particle
// becomes BOTH (bit 1); it counts for the member when a neighbour is a
// non-empty NONE bucket that is not UNDERGROUND.  1 -> 3 leaves every
// "== 0" test unchanged, so the order of the buckets does not matter.
__global__ void k_scan_outside(const Geo* __restrict__ geo, const uint16_t* __restrict__ bmember, Dev A,
                               const uint32_t* __restrict__ cs_all, uint8_t* __restrict__ binv,
                               const uint8_t* __restrict__ bflags, const int8_t* __restrict__ bface, int nbk,
                               int explicit_types, int* __restrict__ adapt) {
  const int gb = blockIdx.x * blockDim.x + threadIdx.x;
  if (gb >= nbk || binv[gb] != PLUME_BINV_POTENTIAL) return;
  const int m = bmember[gb];
  const Geo& g = geo[m];
  const int b = gb - g.bucket_base;
  const uint32_t* cs = cs_all + g.cell_base;
  bool inv = false;
  for_bucket_rows(g, cs, b, [&](uint32_t j0, uint32_t j1) {
    for (uint32_t j = j0; j < j1 && !inv; j++) inv = A.inv[j] == 2;
  });
  if (!inv) return;
  binv[gb] = PLUME_BINV_BOTH;
  const bool grows = any_neighbour(g, b, [&](int nb) {
    const int gn = g.bucket_base + nb;
    const uint8_t f = bflags ? bflags[gn] : 0;
    const int8_t* fi = bface ? bface + 6 * (size_t)gn : nullptr;
    return binv[gn] == PLUME_BINV_NONE && btype_of(f, fi, explicit_types) != 1 && bucket_count(g, cs, nb) > 0;
  });
  if (grows) atomicAdd(adapt + m, 1);
}

// adapt_domain, buckets: a non-empty NONE bucket, neither UNDERGROUND nor
// PRESS_BC, next to a bucket with involved particles becomes POTENTIAL and
// stops absorbing (converted buckets get bit 1 clear, so the tests of the
// other buckets do not see them change)
__global__ void k_adapt_buckets(const Geo* __restrict__ geo, const uint16_t* __restrict__ bmember,
                                const uint32_t* __restrict__ cs_all, uint8_t* __restrict__ binv,
                                uint8_t* __restrict__ bflags, const int8_t* __restrict__ bface, int nbk,
                                int explicit_types, uint8_t* __restrict__ mark) {
  const int gb = blockIdx.x * blockDim.x + threadIdx.x;
  if (gb >= nbk) return;
  mark[gb] = 0;
  if (binv[gb] != PLUME_BINV_NONE) return;
  const int m = bmember[gb];
  const Geo& g = geo[m];
  const int b = gb - g.bucket_base;
  const uint8_t f = bflags ? bflags[gb] : 0;
  const int t = btype_of(f, bface ? bface + 6 * (size_t)gb : nullptr, explicit_types);
  if (t == 1 || t == 2) return;
  const uint32_t* cs = cs_all + g.cell_base;
  if (bucket_count(g, cs, b) == 0) return;
  if (!any_neighbour(g, b, [&](int nb) { return (binv[g.bucket_base + nb] & PLUME_BINV_INVOLVED) != 0; })) return;
  mark[gb] = 1;
  binv[gb] = PLUME_BINV_POTENTIAL;
  if (bflags) bflags[gb] = f & (uint8_t)~PLUME_BUCKET_ABSORBING;
}

// ---- add_pressure_ghost (add_pressure_ghost.cc:37-316): pressure-ghost
// layers around the buckets an adaptation made potentially involved.
// Hydrostatic air of ATMOSPHERE_TYPE 1 (air_prop_hydro, sph_lib.cc:488-592)
struct Atm {
  double Ta0, pa0, Ra, gamma, H1, H2, H3, miu1, miu2, Ata1, Ate1, Ata2, Atb2, Ata3, Atb3, AtC3, Ate3;
};
__device__ __forceinline__ double atm_T(const Atm& a, double h) {
  if (h < 0) return a.Ta0;
  if (h < a.H1) return a.Ta0 - a.miu1 * h;
  if (h < a.H2) return a.Ta0 - a.miu1 * a.H1;
  return a.Ta0 - a.miu1 * a.H1 + a.miu2 * (h - a.H2);
}
__device__ __forceinline__ double atm_p(const Atm& a, double h) {
  if (h < 0) return a.pa0;
  if (h < a.H1) return a.Ata1 * pow(a.Ta0 - a.miu1 * h, a.Ate1);
  if (h < a.H2) return a.Ata2 * exp(a.Atb2 * h);
  return a.AtC3 * pow(a.Atb3 * h + a.Ata3, a.Ate3);
}

// lattice of a bucket: points per axis (C round of edge / dx) at corner +
// dx/2 + i dx, restricted to the z layers [k0, k1)
struct PgLattice {
  double lo[3];
  int n[3], k0, k1;
  __device__ __forceinline__ uint32_t count() const { return (uint32_t)n[0] * (uint32_t)n[1] * (uint32_t)(k1 - k0); }
  __device__ __forceinline__ double zk(int k, double dx) const { return lo[2] + 0.5 * dx + k * dx; }
};
__device__ __forceinline__ PgLattice pg_lattice(const Geo& g, int b, double dx) {
  const int ijk[3] = {b % g.nb[0], (b / g.nb[0]) % g.nb[1], b / (g.nb[0] * g.nb[1])};
  PgLattice L;
  for (int a = 0; a < 3; a++) {
    L.lo[a] = g.mind[a] + ijk[a] * g.del;
    const double hi = g.mind[a] + (ijk[a] + 1) * g.del;
    L.n[a] = (int)round((hi - L.lo[a]) / dx);
  }
  L.k0 = 0;
  L.k1 = L.n[2];
  return L;
}
// points above the ground plane only (add_pressure_ghost.cc:165)
__device__ __forceinline__ void pg_above(PgLattice& L, double dx, double ground) {
  while (L.k0 < L.k1 && !(L.zk(L.k0, dx) > ground)) L.k0++;
}
// points below the ground plane only (add_wall_ghost.cc:165)
__device__ __forceinline__ void pg_below(PgLattice& L, double dx, double ground) {
  int k = 0;
  while (k < L.n[2] && L.zk(k, dx) < ground) k++;
  L.k1 = k;
}

// The lattices a bucket fills.  kind 0, add_pressure_ghost
// (add_pressure_ghost.cc:107-300): a NONE bucket that holds no pressure
// ghost and has a neighbour whose state is not NONE is made active and fills
// its lattice (on-ground MIXED: above the ground; UNDERGROUND: nothing).
// kind 1, add_wall_ghost (add_wall_ghost.cc:124-285): an on-ground MIXED
// bucket that holds particles but no wall ghost fills its lattice below the
// ground, and the bucket below it is made active and filled whole.  kind
// 2, add_air: below.  Returns the number of lattices (0..2).
__device__ __forceinline__ int pg_select(const Geo& g, const Dev& A, const uint32_t* __restrict__ cs,
                                         const uint8_t* __restrict__ binv, const uint8_t* __restrict__ bflags,
                                         const int8_t* __restrict__ bface, int explicit_types, int kind, int b,
                                         double dx, double ground, PgLattice* L, int* activate) {
  *activate = -1;
  const uint8_t f = bflags ? bflags[b] : 0;
  const int8_t* fi = bface ? bface + 6 * (size_t)b : nullptr;
  const int t = btype_of(f, fi, explicit_types);
  const bool onground = t == 3 && fi && fi[4] == -1;
  if (kind == 2) {
    // add_air (add_air.cc:490-795): an empty bucket whose state is not NONE
    // is made active; MIXED and OVERGROUND buckets fill their lattice (on
    // or below the ground: above the ground plane only)
    if (binv[b] == PLUME_BINV_NONE || bucket_count(g, cs, b) > 0) return 0;
    *activate = b;
    if (t != 3 && t != 4) return 0;
    L[0] = pg_lattice(g, b, dx);
    if (onground) pg_above(L[0], dx, ground);
    return 1;
  }
  const uint8_t ghost = kind == 0 ? PLUME_BC_PRESSURE : PLUME_BC_WALL;
  if (kind == 0 && binv[b] != PLUME_BINV_NONE) return 0;
  if (kind == 1 && !onground) return 0;
  bool has = false;
  uint32_t rows = 0;
  for_bucket_rows(g, cs, b, [&](uint32_t j0, uint32_t j1) {
    rows += j1 - j0;
    for (uint32_t j = j0; j < j1 && !has; j++) has = A.bc[j] == ghost;
  });
  if (has) return 0;
  if (kind == 0) {
    if (!any_neighbour(g, b, [&](int nb) { return binv[nb] != PLUME_BINV_NONE; })) return 0;
    *activate = b;
    if (t == 1) return 0;  // UNDERGROUND: none
    L[0] = pg_lattice(g, b, dx);
    if (onground) pg_above(L[0], dx, ground);
    return 1;
  }
  if (rows == 0) return 0;
  L[0] = pg_lattice(g, b, dx);
  pg_below(L[0], dx, ground);
  const int down = b - g.nb[0] * g.nb[1];
  if (down < 0) return 1;
  *activate = down;
  L[1] = pg_lattice(g, down, dx);
  return 2;
}

// One thread per bucket: the count of its lattices; buckets to make active
__global__ void k_pg_buckets(const Geo* __restrict__ geo, Dev A, const uint32_t* __restrict__ cs,
                             const uint8_t* __restrict__ binv, uint8_t* __restrict__ bflags,
                             const int8_t* __restrict__ bface, int nbk, int explicit_types, int kind, double dx,
                             double ground, uint32_t* __restrict__ cnt) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbk) return;
  PgLattice L[2];
  int act;
  const int nl = pg_select(geo[0], A, cs, binv, bflags, bface, explicit_types, kind, b, dx, ground, L, &act);
  uint32_t c = 0;
  for (int q = 0; q < nl; q++) c += L[q].count();
  cnt[b] = c;
  // the activated bucket is b itself (kind 0) or the one below an on-ground
  // bucket (kind 1), which no other bucket activates; selection reads no
  // activity bit, so the order of the writes does not matter
  if (act >= 0 && bflags) bflags[act] &= (uint8_t)~PLUME_BUCKET_INACTIVE;
}

// One block per bucket: its points, lattice by lattice, k fastest, appended
// at row base + offs[b]; state of initial_air (sph_lib.cc:831-866) and the EOS
__global__ void k_pg_fill(const Geo* __restrict__ geo, const Opt* __restrict__ mopt, Dev A,
                          const uint32_t* __restrict__ cs, const uint8_t* __restrict__ binv,
                          const uint8_t* __restrict__ bflags, const int8_t* __restrict__ bface, int explicit_types,
                          int kind, const uint32_t* __restrict__ cnt, const unsigned long long* __restrict__ offs,
                          Atm atm, double dx, double ground, size_t base, unsigned long long key_base) {
  const int b = blockIdx.x;
  const uint32_t nq = cnt[b];
  if (nq == 0) return;
  const Geo& g = geo[0];
  const Opt& o = mopt[0];
  PgLattice L[2];
  int act;
  const int nl = pg_select(g, A, cs, binv, bflags, bface, explicit_types, kind, b, dx, ground, L, &act);
  const uint32_t c0 = nl > 0 ? L[0].count() : 0;
  const double dx2 = 0.5 * dx, s2 = 0.5 * dx;
  const uint8_t bc = kind == 0 ? PLUME_BC_PRESSURE : (kind == 1 ? PLUME_BC_WALL : PLUME_BC_REAL);
  const uint8_t inv = kind == 2 ? 1 : 0;  // add_air: potentially involved
  for (uint32_t q = threadIdx.x; q < nq; q += blockDim.x) {
    const bool second = q >= c0;
    const PgLattice& M = second ? L[1] : L[0];
    const uint32_t u = second ? q - c0 : q;
    const uint32_t nk = (uint32_t)(M.k1 - M.k0);
    const uint32_t i = u / ((uint32_t)M.n[1] * nk);
    const uint32_t j = (u / nk) % (uint32_t)M.n[1];
    const uint32_t k = (uint32_t)M.k0 + u % nk;
    const double x = M.lo[0] + dx2 + i * dx;
    const double y = M.lo[1] + dx2 + j * dx;
    const double z = M.lo[2] + dx2 + k * dx;
    const double T = atm_T(atm, z);
    const double p0 = atm_p(atm, z);
    const double rho = p0 / (atm.Ra * T);
    const double e = p0 / (rho * (atm.gamma - 1));
    const double z1 = z - s2, z2 = z + s2;
    const double d1 = atm_p(atm, z1) / (atm.Ra * atm_T(atm, z1));
    const double d2 = atm_p(atm, z2) / (atm.Ra * atm_T(atm, z2));
    const double vol = ((x + s2) - (x - s2)) * ((y + s2) - (y - s2)) * (z2 - z1);
    const double mass = vol * (0.1666667 * d1 + 0.6666666 * rho + 0.1666667 * d2);
    const size_t r = base + offs[b] + q;
    A.key[r] = key_base + offs[b] + q;
    A.x[r] = x; A.y[r] = y; A.z[r] = z;
    A.vx[r] = 0; A.vy[r] = 0; A.vz[r] = 0;
    A.vsx[r] = 0; A.vsy[r] = 0; A.vsz[r] = 0;
    A.mass[r] = mass; A.h[r] = dx; A.rho[r] = rho; A.e[r] = e; A.Y[r] = 0;
    double gam, p, c, temp, cp = 0;
    eos(o, rho, 0.0, e, gam, p, c, temp, cp, o.lans != 0);
    A.gam[r] = gam; A.p[r] = p; A.c[r] = c; A.T[r] = temp; A.cp[r] = cp;
    A.phase[r] = 1; A.bc[r] = bc; A.inv[r] = inv;
    A.mem[r] = 0; A.bkt[r] = second ? b - g.nb[0] * g.nb[1] : b;
  }
}

// setup_erupt (setup_erupt.cc:44-388): particles other than erupt ghosts
// inside the duct (x^2 + y^2 <= r^2, z in [z_bot, z_top]) are removed
__global__ void k_duct_remove(Dev A, const int* __restrict__ d_count, double r2, double zbot, double ztop,
                              unsigned int* __restrict__ removed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count) return;
  const uint8_t bc = A.bc[i];
  if (bc == BC_DEAD || bc == PLUME_BC_ERUPT) return;
  const double x = A.x[i], y = A.y[i], z = A.z[i];
  if (x * x + y * y <= r2 && z <= ztop && z >= zbot) {
    A.bc[i] = BC_DEAD;
    atomicAdd(removed, 1u);
  }
}

// the duct's erupt ghosts: point q of z layer iz is (xy[2 q], xy[2 q + 1],
// zs[iz]); state of the erupt-ghost constructor (particle.cc:210-316)
__global__ void k_duct_fill(const Opt* __restrict__ mopt, Dev A, const double* __restrict__ xy, int npairs,
                            const double* __restrict__ zs, int nz, PlumeDuct duct, double mass, double sml,
                            size_t base, unsigned long long key_base) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npairs * nz) return;
  const Opt& o = mopt[0];
  const int iz = t / npairs, q = t % npairs;
  const double x = xy[2 * q], y = xy[2 * q + 1];
  const size_t r = base + (size_t)t;
  A.key[r] = key_base + (unsigned long long)t;
  A.x[r] = x; A.y[r] = y; A.z[r] = zs[iz];
  const double dist = x * x + y * y;
  A.vx[r] = 0; A.vy[r] = 0;
  A.vz[r] = duct.profile == 0 ? duct.u_avg : duct.u_avg * 2 * (1 - dist / (duct.radius * duct.radius));
  A.vsx[r] = 0; A.vsy[r] = 0; A.vsz[r] = 0;
  A.mass[r] = mass; A.h[r] = sml; A.rho[r] = duct.rho; A.e[r] = duct.e; A.Y[r] = 1.0;
  double gam, p, c, temp, cp = 0;
  eos(o, duct.rho, 1.0, duct.e, gam, p, c, temp, cp, o.lans != 0);
  A.T[r] = temp; A.cp[r] = cp;
  A.p[r] = duct.p; A.c[r] = duct.c; A.gam[r] = duct.gamma;
  A.phase[r] = 2; A.bc[r] = PLUME_BC_ERUPT; A.inv[r] = 0;
  A.mem[r] = 0; A.bkt[r] = 0;
}

// search_bnd_images (bnd_image.cc:36-245) for a flat ground: a wall ghost
// of a MIXED bucket whose own bucket or one of its 26 neighbours is an
// on-ground MIXED bucket (bottom face below the ground, top face not,
// bucket.h:524-527) is mirrored in the ground plane, image = 2 intsct - x
// with intsct = (x, y, z_ground) (Bucket::calc_intersection_ground for flat
// ground, bucket.cc:346-354); ghosts farther from the ground than the
// domain's height are skipped (bnd_image.cc:146-150)
__global__ void k_find_images(const Geo* __restrict__ geo, Dev A, const int* __restrict__ d_count,
                              const uint8_t* __restrict__ bflags, const int8_t* __restrict__ bface,
                              int explicit_types, double zmax_dist, unsigned long long* __restrict__ okey,
                              double* __restrict__ oxyz, unsigned int* __restrict__ ocount, unsigned int cap) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count || A.bc[i] != PLUME_BC_WALL) return;
  const Geo& g = geo[0];
  const int b = A.bkt[i];
  auto onground_mixed = [&](int q) {
    const uint8_t f = bflags ? bflags[q] : 0;
    const int8_t* fi = bface ? bface + 6 * (size_t)q : nullptr;
    return btype_of(f, fi, explicit_types) == 3 && fi && fi[4] == -1 && fi[5] == 0;
  };
  {
    const uint8_t f = bflags ? bflags[b] : 0;
    if (btype_of(f, bface ? bface + 6 * (size_t)b : nullptr, explicit_types) != 3) return;
  }
  if (!onground_mixed(b) && !any_neighbour(g, b, onground_mixed)) return;
  const double zg = g.lo[2];
  const double z = A.z[i];
  if (fabs(z - zg) > zmax_dist) return;
  const unsigned int slot = atomicAdd(ocount, 1u);
  if (slot >= cap) return;
  okey[slot] = A.key[i];
  oxyz[3 * (size_t)slot] = A.x[i];
  oxyz[3 * (size_t)slot + 1] = A.y[i];
  oxyz[3 * (size_t)slot + 2] = 2 * zg - z;
}

// adapt_domain, particles of the converted buckets: real (100) and
// potentially involved (1) -- on-ground MIXED buckets their pressure ghosts,
// other MIXED buckets those inside the domain (determine_escape), OVERGROUND
// buckets every particle
__global__ void k_adapt_particles(const Geo* __restrict__ geo, Dev A, const int* __restrict__ d_count,
                                  const uint8_t* __restrict__ mark, const uint8_t* __restrict__ bflags,
                                  const int8_t* __restrict__ bface, int explicit_types) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count) return;
  const uint8_t bc = A.bc[i];
  if (bc == BC_DEAD) return;
  const Geo& g = geo[A.mem[i]];
  const int gb = g.bucket_base + A.bkt[i];
  if (!mark[gb]) return;
  const uint8_t f = bflags ? bflags[gb] : 0;
  const int8_t* fi = bface ? bface + 6 * (size_t)gb : nullptr;
  const int t = btype_of(f, fi, explicit_types);
  bool turn = true;
  if (t == 3 && fi && fi[4] == -1) {
    turn = bc == PLUME_BC_PRESSURE;
  } else if (t == 3) {
    const double pos[3] = {A.x[i], A.y[i], A.z[i]};
    bool esc = false;
    for (int a = 0; a < 3 && fi; a++) {
      if (fi[2 * a] == -1) {
        if ((pos[a] - g.lo[a]) < -TINY_D) esc = true;
      } else if (fi[2 * a + 1] == 1) {
        if ((pos[a] - g.hi[a]) > TINY_D) esc = true;
      }
    }
    turn = !esc;
  }
  if (turn) {
    A.bc[i] = PLUME_BC_REAL;
    A.inv[i] = 1;
  }
}

// ---- eruption inlet (add_new_erupt, setup_erupt.cc:389-673) ---------------
struct Inlet {
  const double* xy;   // column positions (2 per column)
  const double* vel;  // column inflow velocity
  int ncol;
  double bot, spacing, mass, h, rho, e, p, gam, c, Y;
  uint64_t key_base;
};
// One thread per duct column, while iferupt: the particles the flow has made
// room for since the previous step enter at the duct bottom, spaced by
// `spacing` along the column, with the vent state (the Particle constructor
// of particle.cc:210-316: v = (0, 0, vel), Y = 1, phase 2, EOS for T and
// cp, then p, c and gamma set to the vent values).  New particles take the
// dead rows after the live ones (row counter, at most `reserve` a step);
// the key of a column's k-th particle is key_base + k ncol + column.
__global__ void k_inject(Inlet in, const Opt* __restrict__ mopt, Dev A, const int* __restrict__ d_count,
                         TimeState* ts, unsigned long long* __restrict__ colcnt, int* __restrict__ rowctr,
                         int reserve, int cap_rows) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= in.ncol || !ts->erupt) return;
  const Opt& o = mopt[0];
  const double dt = ts->dtime;
  const double t_total = ts->time - dt;
  const double vel = in.vel[col];
  const double t_each = in.spacing / vel;
  double t_add = fmod(t_total, t_each) + dt;
  const int nn = (int)floor(t_add / t_each);
  t_add = t_add - nn * t_each;
  for (int i = 0; i < nn; i++) {
    const int r = atomicAdd(rowctr, 1);
    const int row = *d_count + r;
    if (r >= reserve || row >= cap_rows) {
      set_status(ts, 5);
      return;
    }
    const unsigned long long k = colcnt[col]++;
    A.key[row] = in.key_base + k * (unsigned long long)in.ncol + (unsigned long long)col;
    A.x[row] = in.xy[2 * col];
    A.y[row] = in.xy[2 * col + 1];
    A.z[row] = in.bot + (t_add + i * t_each) * vel;
    A.vx[row] = 0; A.vy[row] = 0; A.vz[row] = vel;
    A.vsx[row] = 0; A.vsy[row] = 0; A.vsz[row] = 0;
    A.mass[row] = in.mass;
    A.h[row] = in.h;
    A.rho[row] = in.rho;
    A.e[row] = in.e;
    A.Y[row] = in.Y;
    A.phase[row] = 2;
    A.bc[row] = 0;
    A.inv[row] = 0;
    A.bkt[row] = 0;
    A.mem[row] = 0;
    double gam, p, c, temp, cp = 0.;
    eos(o, in.rho, in.Y, in.e, gam, p, c, temp, cp, o.lans != 0);
    A.T[row] = temp;
    A.cp[row] = cp;
    A.p[row] = in.p;
    A.c[row] = in.c;
    A.gam[row] = in.gam;
  }
}
// the injected rows join the counted rows
__global__ void k_inject_count(int* d_count, const int* __restrict__ rowctr, int reserve) {
  *d_count += min(*rowctr, reserve);
}
__global__ void k_mark_dead(uint8_t* bc, size_t from, size_t to) {
  const size_t r = from + blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (r < to) bc[r] = BC_DEAD;
}

}  // namespace

// ============================================================================
// context
// ============================================================================
static thread_local std::string g_create_error;

// Adjoint (plume_adjoint_record / plume_adjoint_backward): one step of a
// recomputed segment, as the backward of the step reads it (sorted order of
// the step).
struct AdjRec {
  Dev S;                                 // state after the sort, before adaptive h
  double *h1, *hit;                      // h after adaptive h; its iterates
  uint8_t* nit;
  double *v1x, *v1y, *v1z, *e1;          // after the momentum commit
  double *rho2, *Y2, *e2;                // after the density commit
  double *vs3x, *vs3y, *vs3z;            // after the LANS filter
  double *wnd, *wnv;                     // filter normalisations
  uint8_t* bc3;                          // bc after the position update
  uint32_t* perm;                        // sorted row -> row before the sort
  NList L;
  uint32_t* real_idx;
  int* d_real;
  uint32_t* cs;
  double* h27;
  TimeState* ts;                         // time state after the step
  int* argmin;                           // the particle that set dt
  int* d_count;                          // live rows after the sort
  int adaptive;                          // adaptive h ran in this step
};
// state at a checkpoint
struct AdjCkpt {
  Dev A;
  int* d_count;
  TimeState* ts;
  size_t n_alloc;
  int host_step;
};

struct plume_ctx {
  PlumeOptions opt{};  // member 0's options
  Opt o{};             // member 0's options: the fields every member shares
  // ensemble members (one for a single run): grid, options and time state of
  // each, on the host and on the device
  int nmem = 1;
  bool batch = false;
  std::vector<Geo> hgeo;
  std::vector<Opt> hopt;
  Geo* d_geo = nullptr;
  Opt* d_opt = nullptr;
  uint16_t* bmember = nullptr;  // member of every per-bucket table entry
  int* d_hstep = nullptr;       // steps issued (adaptive_sml schedule)
  // CUDA graph of graph_steps steps (plume_batch_run)
  bool capturing = false;
  cudaGraphExec_t gexec = nullptr;
  int gsteps = 0;
  size_t gn = 0;
  unsigned long long glaunches = 0;
  cudaEvent_t run_ev[2] = {nullptr, nullptr};  // device time of plume_batch_run
  cudaStream_t st = nullptr;
  size_t cap = 0;
  size_t n_alloc = 0;  // rows in use (upper bound of live particles)
  Dev A{}, B{};
  Work W{};
  Packed K{};  // FP32 pair records of the mixed path
  NList L{};   // per-step masked neighbour lists (3D)
  bool use_lists = true;
  // compacted need_neigh indices of the step (3D list sweeps)
  unsigned int* rflag = nullptr;
  unsigned long long *roffs = nullptr, *rsums = nullptr, *rtot = nullptr;
  uint32_t* real_idx = nullptr;
  int* d_real = nullptr;
  // 3D sweep walk: one warp per particle (true) or one thread per particle;
  // default per precision, PLUME_SWEEP=warp|thread overrides
  bool sweep_warp = false;
  bool list_warp = false;  // mixed list sweeps: one warp per particle (k_sweep3_wl), opt-in
  uint32_t *keys = nullptr, *perm = nullptr, *cs = nullptr;
  uint32_t ncells = 0;
  int keybits = 1;
  int* d_count = nullptr;
  TimeState* ts = nullptr;    // nmem entries
  TimeState* h_ts = nullptr;  // pinned mirror
  unsigned long long* hb = nullptr;
  double* h27 = nullptr;
  int nbk = 1;
  uint8_t* bflags = nullptr;
  int8_t* bface = nullptr;
  RadixSorter sorter;
  std::vector<void*> allocs;
  int host_step = 0;
  bool pending_dead = false;  // row order unknown: search before row-order reads
  bool has_dead = false;      // rows deleted by the last steps are still in the table
  unsigned long long* d_nreal = nullptr;  // plume_count's real-particle count
  // output snapshot: staging arrays (lazily sized), side stream, events
  Dev snap{};
  size_t snap_cap = 0, snap_n = 0;
  cudaStream_t snap_st = nullptr;
  cudaEvent_t snap_staged = nullptr, snap_done = nullptr;
  bool snap_busy = false;
  TimeState* snap_ts = nullptr;  // pinned: time and step at the snapshot
  std::string err;
  // per-step event sets (NEV events each) for the phase times of a call
  std::vector<cudaEvent_t> evs;
  cudaEvent_t* ev = nullptr;  // event set of the step being issued
  float phase_ms[NPHASE] = {};
  unsigned long long launches = 0;
  // adjoint
  AdjRec* rec = nullptr;        // snapshot target of the step being issued
  std::vector<AdjRec> recs;     // one per step of a segment
  std::vector<AdjCkpt> ckpts;   // every adj_every steps, then the final state
  std::vector<void*> adj_allocs;
  int adj_every = 0, adj_steps = 0;
  size_t adj_rows = 0;
  // wall images (plume_set_wall_images), sorted by ghost key
  uint64_t* img_key = nullptr;
  double* img_xyz = nullptr;
  int nimg = 0;
  int* bc_map = nullptr;  // row of (member, image), -1 when absent
  // tile order of the list sweeps (single 3D runs with lists)
  int ntiles = 0;
  unsigned int* tcount = nullptr;
  unsigned long long *toffs = nullptr, *tsums = nullptr, *ttot = nullptr;
  uint32_t* real_tile = nullptr;
  int* d_real_tile = nullptr;
  // domain growth: involvement state per bucket, the scan's count per
  // member, buckets converted by the last adapt_domain
  uint8_t* binv = nullptr;
  int* d_adapt = nullptr;
  uint8_t* bmark = nullptr;
  int explicit_types = 0;
  // GSPH gradients of the last step ((D+2)*D doubles per row; GSPH only)
  double* grad = nullptr;
  bool grad_valid = false;
  // eruption inlet (plume_set_inlet)
  Inlet inlet{};
  double* inlet_buf = nullptr;              // column xy + vel
  unsigned long long* inlet_colcnt = nullptr;
  int* inlet_rowctr = nullptr;
  int inlet_reserve = 0;
};

// device scratch of one call, freed on every return path
struct ScratchFree {
  void* p[4] = {nullptr, nullptr, nullptr, nullptr};
  ~ScratchFree() {
    for (void* q : p)
      if (q) cudaFree(q);
  }
};

#define CK(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                  \
      return PLUME_E_CUDA;                                                            \
    }                                                                                 \
  } while (0)

static int dev_alloc(plume_ctx* ctx, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    ctx->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return PLUME_E_CUDA;
  }
  ctx->allocs.push_back(*p);
  return PLUME_OK;
}
#define DALLOC(ptr, bytes)                                                   \
  do {                                                                       \
    int rc_ = dev_alloc(ctx, (void**)&(ptr), (bytes));                       \
    if (rc_) return rc_;                                                     \
  } while (0)

static int alloc_dev(plume_ctx* ctx, Dev& D, size_t cap) {
  DALLOC(D.key, 8 * cap);
  double** f[] = {&D.x, &D.y, &D.z, &D.vx, &D.vy, &D.vz, &D.vsx, &D.vsy, &D.vsz, &D.mass,
                  &D.h, &D.rho, &D.e, &D.p, &D.Y, &D.gam, &D.c, &D.T, &D.cp};
  for (auto p : f) DALLOC(*p, 8 * cap);
  DALLOC(D.phase, cap);
  DALLOC(D.bc, cap);
  DALLOC(D.inv, cap);
  DALLOC(D.bkt, 4 * cap);
  DALLOC(D.mem, 2 * cap);
  return PLUME_OK;
}

static Opt make_opt(const PlumeOptions& p) {
  Opt o;
  o.dim = p.dim; o.prec = p.precision; o.kernel = p.kernel; o.lans = p.lans; o.esmooth = p.energy_smooth;
  o.pgc = p.pghost_contrib; o.adaptive = p.adaptive_sml; o.interval = p.sml_interval > 0 ? p.sml_interval : 1;
  o.num_loop = p.num_loop; o.thresh = p.thresh; o.c_smooth = p.c_smooth; o.eta = p.eta_smooth;
  o.alpha = p.alpha; o.beta = p.beta; o.ata = p.ata; o.cfl = p.cfl; o.cutoff2 = p.cutoff2;
  o.list_factor = p.list_factor; o.g = p.g; o.ng0 = p.ng0; o.cvs = p.cvs; o.cvg = p.cvg; o.cva = p.cva;
  o.rg = p.rg; o.ra = p.ra; o.vent_z = p.vent_z; o.sml2 = p.sml_phase2; o.max_time = p.max_time;
  o.timeoutput = p.timeoutput; o.stat_erupt = p.stat_erupt; o.end_erupt = p.end_erupt;
  o.ksupport = (p.kernel == PLUME_KERNEL_M4) ? 2.0 : 3.0;
  o.max_steps = p.max_steps;
  o.method = p.method;
  o.gsph_solver = p.gsph_solver;
  o.gsph_recon = p.gsph_recon;
  o.gsph_vol = p.gsph_vol;
  o.gsph_mono = p.gsph_mono;
  o.gsph_wave = p.gsph_wave_speed;
  return o;
}

// waits for the stream, mirrors the members' time states and returns the
// first member's nonzero status (cleared on the device).  An ensemble keeps
// its members' statuses: a failed member stops, the others go on, and
// plume_batch_time reports them.
static int ctx_sync_status(plume_ctx* ctx) {
  CK(cudaStreamSynchronize(ctx->st));
  CK(cudaMemcpy(ctx->h_ts, ctx->ts, sizeof(TimeState) * ctx->nmem, cudaMemcpyDeviceToHost));
  if (ctx->batch) return PLUME_OK;
  int s = 0;
  for (int m = 0; m < ctx->nmem; m++) {
    const int sm = ctx->h_ts[m].status;
    if (!sm) continue;
    if (!s) {
      s = sm;
      ctx->err = std::string("device status ") + std::to_string(sm) +
                 (ctx->nmem > 1 ? std::string(" in member ") + std::to_string(m) : std::string());
    }
    TimeState clr = ctx->h_ts[m];
    clr.status = 0;
    CK(cudaMemcpy(ctx->ts + m, &clr, sizeof(TimeState), cudaMemcpyHostToDevice));
  }
  return s;
}

static void record_ev(plume_ctx* ctx, int k) {
  if (!ctx->capturing) cudaEventRecord(ctx->ev[k], ctx->st);
}

__global__ void k_set_int(int* p, int v) { *p = v; }

static void dcopy(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st);
}
// every particle array of a Dev, rows [0, n)
static void copy_dev(const Dev& d, const Dev& s, size_t n, cudaStream_t st) {
  dcopy(d.key, s.key, 8 * n, st);
  double* const dd[19] = {d.x, d.y, d.z, d.vx, d.vy, d.vz, d.vsx, d.vsy, d.vsz, d.mass,
                          d.h, d.rho, d.e, d.p, d.Y, d.gam, d.c, d.T, d.cp};
  double* const ss[19] = {s.x, s.y, s.z, s.vx, s.vy, s.vz, s.vsx, s.vsy, s.vsz, s.mass,
                          s.h, s.rho, s.e, s.p, s.Y, s.gam, s.c, s.T, s.cp};
  for (int f = 0; f < 19; f++) dcopy(dd[f], ss[f], 8 * n, st);
  dcopy(d.phase, s.phase, n, st);
  dcopy(d.bc, s.bc, n, st);
  dcopy(d.inv, s.inv, n, st);
  dcopy(d.bkt, s.bkt, 4 * n, st);
  dcopy(d.mem, s.mem, 2 * n, st);
}

// adjoint snapshots of the step being issued (ctx->rec set)
static void snap_search(plume_ctx* ctx) {
  AdjRec* r = ctx->rec;
  const size_t n = ctx->n_alloc;
  cudaStream_t st = ctx->st;
  copy_dev(r->S, ctx->A, n, st);
  dcopy(r->perm, ctx->perm, 4 * n, st);
  dcopy(r->d_count, ctx->d_count, sizeof(int), st);
  k_set_int<<<1, 1, 0, st>>>(r->argmin, 0x7fffffff);
  k_dt_argmin<<<nblocks(n ? n : 1), NTHREADS, 0, st>>>(ctx->A, ctx->d_count, ctx->ts, r->argmin);
}

// search: keys, radix sort, gather into B, swap, cell_start
static int search(plume_ctx* ctx) {
  const int n = (int)ctx->n_alloc;
  cudaStream_t st = ctx->st;
  if (n == 0) {
    k_fill_cs<<<nblocks((size_t)ctx->ncells + 2, 256), 256, 0, st>>>(ctx->cs, ctx->ncells, ctx->d_count);
    ctx->launches++;
    return PLUME_OK;
  }
  k_keys<<<nblocks(n), NTHREADS, 0, st>>>(ctx->d_geo, ctx->A, n, ctx->keys, ctx->ncells, ctx->ts);
  ctx->launches++;
  ctx->launches += ctx->sorter.sort(ctx->keys, ctx->perm, n, ctx->keybits, st);
  k_gather<<<nblocks(n), NTHREADS, 0, st>>>(ctx->d_geo, ctx->A, ctx->B, ctx->W, ctx->perm, n);
  std::swap(ctx->A, ctx->B);
  k_cell_start<<<nblocks((size_t)ctx->ncells + 2, 256), 256, 0, st>>>(ctx->keys, n, ctx->ncells, ctx->cs, ctx->d_count);
  ctx->launches += 2;
  ctx->pending_dead = false;
  ctx->has_dead = false;
  if (ctx->rec) snap_search(ctx);
  if (ctx->inlet_reserve) {
    // rows the inlet may fill this step: dead until it does
    const size_t to = std::min(ctx->cap, (size_t)n + (size_t)ctx->inlet_reserve);
    if (to > (size_t)n)
      k_mark_dead<<<nblocks(to - (size_t)n, 256), 256, 0, st>>>(ctx->A.bc, (size_t)n, to);
  }
  CK(cudaGetLastError());
  return PLUME_OK;
}

// GSPH momentum: calc_gradients (when the states read them, or always
// with gsph_gradients), then the two-pass Riemann sweep
template <int D, typename T>
static void launch_gsph(plume_ctx* ctx, int nb) {
  cudaStream_t st = ctx->st;
  const bool recon = ctx->o.gsph_recon != PLUME_RECON_ZEROTH;
  ctx->grad_valid = recon || ctx->opt.gsph_gradients;
  if (ctx->grad_valid) {
    k_gsph_grad<D, T><<<nb, NTHREADS, 0, st>>>(ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->d_count,
                                               ctx->ts, ctx->grad);
    ctx->launches++;
  }
  k_gsph_mom<D, T><<<nb, NTHREADS, 0, st>>>(ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->h27, ctx->d_count,
                                            ctx->ts, recon ? ctx->grad : nullptr);
}

// The compacted need_neigh particles of the stepping members: in sorted
// order (the list build's order) and, for single runs, tile by tile (the
// sweeps' order).  They depend on the particle types and cells only, so
// they can be formed before the adaptive-h pass.
template <bool MULTI>
static void compact_real(plume_ctx* ctx, int n, int nb, bool tiled) {
  cudaStream_t st = ctx->st;
  const int ns = n ? n : 1, nsb = (ns + 1023) / 1024;
  k_real_flags<<<nb, NTHREADS, 0, st>>>(ctx->A, ctx->d_count, ns, ctx->ts, ctx->rflag);
  k_scan_blocks<<<nsb, 1024, 0, st>>>(ctx->rflag, ns, ctx->roffs, ctx->rsums);
  k_scan_sums<<<1, 1024, 0, st>>>(ctx->rsums, nsb, ctx->rtot);
  k_scan_add<<<nsb, 1024, 0, st>>>(ctx->roffs, ns, ctx->rsums);
  k_real_scatter<<<nb, NTHREADS, 0, st>>>(ctx->rflag, ctx->roffs, ns, ctx->real_idx, ctx->d_real, ctx->rtot);
  ctx->launches += 5;
  if (tiled) {
    const Geo& g0 = ctx->hgeo[0];
    const int ntx = (g0.G[0] + TILE_X - 1) / TILE_X, nty = (g0.G[1] + TILE_Y - 1) / TILE_Y;
    const int nt = ctx->ntiles, ntb = (nt + 1023) / 1024;
    k_tile_count<<<nblocks(nt), NTHREADS, 0, st>>>(g0, ctx->A, ctx->cs, ctx->d_count, ctx->ts, ntx, nty, nt,
                                                   ctx->tcount);
    k_scan_blocks<<<ntb, 1024, 0, st>>>(ctx->tcount, nt, ctx->toffs, ctx->tsums);
    k_scan_sums<<<1, 1024, 0, st>>>(ctx->tsums, ntb, ctx->ttot);
    k_scan_add<<<ntb, 1024, 0, st>>>(ctx->toffs, nt, ctx->tsums);
    k_tile_fill<<<nblocks(nt), NTHREADS, 0, st>>>(g0, ctx->A, ctx->cs, ctx->d_count, ctx->ts, ntx, nty, nt,
                                                  ctx->toffs, ctx->ttot, ctx->real_tile, ctx->d_real_tile);
    ctx->launches += 5;
  }
}

// a list sweep: mixed path one warp per particle, FP64 path one thread
template <typename T, template <typename> class SW, bool MULTI>
static void launch_list_sweep(plume_ctx* ctx, const Geos<MULTI>& gs, int nb, int nbw, const int* cnt,
                              const uint32_t* idx) {
  if (sizeof(T) == 4 && ctx->list_warp)
    k_sweep3_wl<SW, MULTI><<<nbw, NTHREADS, 0, ctx->st>>>(ctx->o, gs, ctx->A, ctx->W, ctx->K, ctx->cs, ctx->h27,
                                                          cnt, idx, ctx->ts, ctx->L);
  else
    k_sweep3_list<T, SW, MULTI><<<nb, NTHREADS, 0, ctx->st>>>(ctx->o, gs, ctx->A, ctx->W, ctx->K, ctx->cs, ctx->h27,
                                                              cnt, idx, ctx->ts, ctx->L);
}

template <int D, typename T, bool MULTI>
static void launch_sweeps(plume_ctx* ctx, bool adaptive_now) {
  const Geos<MULTI> gs{ctx->hgeo[0], ctx->d_geo};
  cudaStream_t st = ctx->st;
  const int n = (int)ctx->n_alloc;
  const int nb = nblocks(n);
  AdjRec* rec = ctx->rec;
  const bool lists = (D == 3) && ctx->use_lists;
  // order of the list sweeps: tile by tile for single runs
  const bool tiled = !MULTI && ctx->ntiles;
  const uint32_t* sweep_idx = tiled ? ctx->real_tile : ctx->real_idx;
  const int* sweep_cnt = tiled ? ctx->d_real_tile : ctx->d_real;
  bool compacted = false;
  const bool adapt = adaptive_now || (ctx->capturing && ctx->o.adaptive);
  if (adapt) {
    // a captured step decides on the device (step counter % interval)
    if (D == 3 && sizeof(T) == 4 && lists && !rec) {
      // mixed 3D: over the compacted particles, packed records
      compact_real<MULTI>(ctx, n, nb, tiled);
      compacted = true;
      k_pack_adapt<<<nb, NTHREADS, 0, st>>>(ctx->A, ctx->K, ctx->W, ctx->o.pgc, ctx->d_count);
      k_adaptive_mixed<MULTI><<<nb, NTHREADS, 0, st>>>(ctx->o, gs, ctx->A, ctx->W, ctx->K, ctx->cs, sweep_cnt,
                                                       sweep_idx, ctx->ts, ctx->d_hstep, ctx->capturing ? 0 : 1);
      ctx->launches += 2;
    } else {
      k_adaptive<D, T><<<nb, NTHREADS, 0, st>>>(ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->d_count, ctx->ts,
                                                ctx->d_hstep, ctx->capturing ? 0 : 1, rec ? rec->hit : nullptr,
                                                rec ? rec->nit : nullptr, n);
      ctx->launches++;
    }
  }
  if (rec) {
    dcopy(rec->h1, ctx->A.h, 8 * (size_t)n, st);
    rec->adaptive = adaptive_now ? 1 : 0;
    ctx->W.wnd = rec->wnd;
    ctx->W.wnv = rec->wnv;
  }
  record_ev(ctx, 3);
  k_hmax_reset<<<nblocks(ctx->nbk, 256), 256, 0, st>>>(ctx->hb, ctx->nbk);
  k_hmax<<<nb, NTHREADS, 0, st>>>(ctx->d_geo, ctx->A, ctx->d_count, ctx->hb, D);
  k_hmax27<<<nblocks(ctx->nbk, 256), 256, 0, st>>>(ctx->d_geo, ctx->bmember, ctx->nbk, ctx->hb, ctx->h27);
  const int nbw = nblocks(n ? n : 1, WP_WARPS);  // one warp per particle
  const bool mixed = sizeof(T) == 4;
  const bool gsph = ctx->o.method != PLUME_METHOD_SPH;  // GSPH or its random choice variant
  if constexpr (D == 3) {
    if (lists) {
      if (!compacted) compact_real<MULTI>(ctx, n, nb, tiled);
      if (mixed) {
        k_pack_pos<<<nb, NTHREADS, 0, st>>>(ctx->A, ctx->K, ctx->W, ctx->d_count);
        ctx->launches++;
      }
      k_build_lists<T, MULTI><<<nb, NTHREADS, 0, st>>>(ctx->o, gs, ctx->A, ctx->W, ctx->K, ctx->cs, ctx->h27,
                                                       ctx->d_real, ctx->real_idx, ctx->ts, ctx->L);
      ctx->launches++;
      if (rec) {
        dcopy(rec->L.e, ctx->L.e, sizeof(uint2) * (size_t)LCAP * n, st);
        dcopy(rec->L.cnt, ctx->L.cnt, sizeof(uint16_t) * (size_t)n, st);
        dcopy(rec->real_idx, ctx->real_idx, 4 * (size_t)n, st);
        dcopy(rec->d_real, ctx->d_real, sizeof(int), st);
        dcopy(rec->cs, ctx->cs, 4 * ((size_t)ctx->ncells + 2), st);
        dcopy(rec->h27, ctx->h27, 8 * (size_t)ctx->nbk, st);
      }
    }
  }
  record_ev(ctx, 4);
  if constexpr (D == 3) {
    if (mixed) {
      k_pack_mom<<<nb, NTHREADS, 0, st>>>(ctx->A, ctx->K, ctx->W, ctx->o.lans, ctx->d_count);
      ctx->launches++;
    }
    record_ev(ctx, 11);
    if (gsph)
      launch_gsph<D, T>(ctx, nb);
    else if (lists)
      launch_list_sweep<T, WMom, MULTI>(ctx, gs, nb, nbw, sweep_cnt, sweep_idx);
    else if (ctx->sweep_warp)
      k_sweep3<T, WMom, true, MULTI><<<nbw, NTHREADS, 0, st>>>(ctx->o, gs, ctx->A, ctx->W, ctx->K, ctx->cs, ctx->h27, ctx->d_count, ctx->ts);
    else
      k_sweep3<T, WMom, false, MULTI><<<nb, NTHREADS, 0, st>>>(ctx->o, gs, ctx->A, ctx->W, ctx->K, ctx->cs, ctx->h27, ctx->d_count, ctx->ts);
  } else {
    record_ev(ctx, 11);
    if (gsph)
      launch_gsph<D, T>(ctx, nb);
    else
      k_momentum<D, T><<<nb, NTHREADS, 0, st>>>(ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->h27, ctx->d_count, ctx->ts);
  }
  record_ev(ctx, 5);
  k_commit_mom<D><<<nb, NTHREADS, 0, st>>>(ctx->d_opt, ctx->A, ctx->W, ctx->d_count, ctx->ts);
  ctx->launches += 5;
  if (rec) {
    dcopy(rec->v1x, ctx->A.vx, 8 * (size_t)n, st);
    dcopy(rec->v1y, ctx->A.vy, 8 * (size_t)n, st);
    dcopy(rec->v1z, ctx->A.vz, 8 * (size_t)n, st);
    dcopy(rec->e1, ctx->A.e, 8 * (size_t)n, st);
  }
  record_ev(ctx, 6);
  if constexpr (D == 3) {
    if (mixed) {
      k_pack_dens<<<nb, NTHREADS, 0, st>>>(ctx->A, ctx->K, ctx->W, ctx->o.pgc, ctx->d_count);
      ctx->launches++;
    }
    if (lists)
      launch_list_sweep<T, WDens, MULTI>(ctx, gs, nb, nbw, sweep_cnt, sweep_idx);
    else if (ctx->sweep_warp)
      k_sweep3<T, WDens, true, MULTI><<<nbw, NTHREADS, 0, st>>>(ctx->o, gs, ctx->A, ctx->W, ctx->K, ctx->cs, ctx->h27, ctx->d_count, ctx->ts);
    else
      k_sweep3<T, WDens, false, MULTI><<<nb, NTHREADS, 0, st>>>(ctx->o, gs, ctx->A, ctx->W, ctx->K, ctx->cs, ctx->h27, ctx->d_count, ctx->ts);
  } else
    k_density<D, T><<<nb, NTHREADS, 0, st>>>(ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->h27, ctx->d_count, ctx->ts);
  record_ev(ctx, 7);
  k_commit_dens<D><<<nb, NTHREADS, 0, st>>>(ctx->d_opt, ctx->A, ctx->W, ctx->d_count, ctx->ts);
  ctx->launches += 2;
  if (rec) {
    dcopy(rec->rho2, ctx->A.rho, 8 * (size_t)n, st);
    dcopy(rec->Y2, ctx->A.Y, 8 * (size_t)n, st);
    dcopy(rec->e2, ctx->A.e, 8 * (size_t)n, st);
  }
  record_ev(ctx, 8);
  if (ctx->o.lans) {
    if constexpr (D == 3) {
      if (mixed) {
        k_pack_vel<<<nb, NTHREADS, 0, st>>>(ctx->A, ctx->K, ctx->W, ctx->d_count);
        ctx->launches++;
      }
      if (lists)
        launch_list_sweep<T, WVel, MULTI>(ctx, gs, nb, nbw, sweep_cnt, sweep_idx);
      else if (ctx->sweep_warp)
        k_sweep3<T, WVel, true, MULTI><<<nbw, NTHREADS, 0, st>>>(ctx->o, gs, ctx->A, ctx->W, ctx->K, ctx->cs, ctx->h27, ctx->d_count, ctx->ts);
      else
        k_sweep3<T, WVel, false, MULTI><<<nb, NTHREADS, 0, st>>>(ctx->o, gs, ctx->A, ctx->W, ctx->K, ctx->cs, ctx->h27, ctx->d_count, ctx->ts);
    } else
      k_velocity<D, T><<<nb, NTHREADS, 0, st>>>(ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->d_count, ctx->ts);
    ctx->launches++;
  }
  if (rec) {
    dcopy(rec->vs3x, ctx->A.vsx, 8 * (size_t)n, st);
    dcopy(rec->vs3y, ctx->A.vsy, 8 * (size_t)n, st);
    dcopy(rec->vs3z, ctx->A.vsz, 8 * (size_t)n, st);
    ctx->W.wnd = nullptr;
    ctx->W.wnv = nullptr;
  }
  record_ev(ctx, 9);
}

// wall boundary on the sorted state (per-bucket maximum h bounds its walk)
static void apply_bc(plume_ctx* ctx) {
  cudaStream_t st = ctx->st;
  const int n = (int)ctx->n_alloc;
  k_hmax_reset<<<nblocks(ctx->nbk, 256), 256, 0, st>>>(ctx->hb, ctx->nbk);
  k_hmax<<<nblocks(n ? n : 1), NTHREADS, 0, st>>>(ctx->d_geo, ctx->A, ctx->d_count, ctx->hb, ctx->o.dim);
  k_hmax27<<<nblocks(ctx->nbk, 256), 256, 0, st>>>(ctx->d_geo, ctx->bmember, ctx->nbk, ctx->hb, ctx->h27);
  const int nslots = ctx->nmem * ctx->nimg;
  cudaMemsetAsync(ctx->bc_map, 0xff, sizeof(int) * (size_t)nslots, st);
  k_bc_map<<<nblocks(n ? n : 1), NTHREADS, 0, st>>>(ctx->A, ctx->d_count, ctx->img_key, ctx->nimg, ctx->bc_map);
  if (ctx->opt.precision == PLUME_PREC_MIXED) {
    k_pack_bc<<<nblocks(n ? n : 1), NTHREADS, 0, st>>>(ctx->A, ctx->K, ctx->W, ctx->d_count);
    k_apply_bcond<float><<<nblocks((size_t)nslots * BCG), NTHREADS, 0, st>>>(ctx->d_opt, ctx->d_geo, ctx->A, ctx->W, ctx->K,
                                                               ctx->cs, ctx->h27, ctx->bc_map, nslots, ctx->nimg,
                                                               ctx->img_xyz, ctx->ts);
    ctx->launches++;
  } else {
    k_apply_bcond<double><<<nblocks((size_t)nslots * BCG), NTHREADS, 0, st>>>(ctx->d_opt, ctx->d_geo, ctx->A, ctx->W, ctx->K,
                                                                ctx->cs, ctx->h27, ctx->bc_map, nslots, ctx->nimg,
                                                                ctx->img_xyz, ctx->ts);
  }
  ctx->launches += 5;
}

// one step, no host synchronisation
static int step_async(plume_ctx* ctx) {
  cudaStream_t st = ctx->st;
  const int n = (int)ctx->n_alloc;
  record_ev(ctx, 0);
  const int mb = nblocks(ctx->nmem);
  k_begin_step<<<mb, NTHREADS, 0, st>>>(ctx->d_opt, ctx->ts, ctx->nmem, ctx->d_hstep);
  k_dt_reduce<<<nblocks(n ? n : 1), NTHREADS, 0, st>>>(ctx->A, ctx->d_count, ctx->ts);
  k_incrtime<<<mb, NTHREADS, 0, st>>>(ctx->d_opt, ctx->ts, ctx->nmem);
  ctx->launches += 3;
  record_ev(ctx, 1);
  int rc = search(ctx);
  if (rc) return rc;
  record_ev(ctx, 13);
  if (ctx->nimg) apply_bc(ctx);
  record_ev(ctx, 2);
  ctx->host_step++;
  bool adaptive_now = ctx->o.adaptive && (ctx->host_step % ctx->o.interval) == 0;
  const bool mixed = ctx->opt.precision == PLUME_PREC_MIXED;
  if (ctx->o.dim == 3) {
    if (ctx->nmem > 1) {
      if (mixed) launch_sweeps<3, float, true>(ctx, adaptive_now); else launch_sweeps<3, double, true>(ctx, adaptive_now);
    } else {
      if (mixed) launch_sweeps<3, float, false>(ctx, adaptive_now); else launch_sweeps<3, double, false>(ctx, adaptive_now);
    }
    k_update_pos<3><<<nblocks(n), NTHREADS, 0, st>>>(ctx->d_opt, ctx->d_geo, ctx->A, ctx->bflags, ctx->bface, ctx->d_count, ctx->ts);
  } else {
    if (mixed) launch_sweeps<1, float, true>(ctx, adaptive_now); else launch_sweeps<1, double, true>(ctx, adaptive_now);
    k_update_pos<1><<<nblocks(n), NTHREADS, 0, st>>>(ctx->d_opt, ctx->d_geo, ctx->A, ctx->bflags, ctx->bface, ctx->d_count, ctx->ts);
  }
  record_ev(ctx, 12);
  if (ctx->inlet_reserve) {  // add_new_erupt (main.cc:416-417)
    cudaMemsetAsync(ctx->inlet_rowctr, 0, sizeof(int), st);
    k_inject<<<nblocks(ctx->inlet.ncol), NTHREADS, 0, st>>>(ctx->inlet, ctx->d_opt, ctx->A, ctx->d_count, ctx->ts,
                                                             ctx->inlet_colcnt, ctx->inlet_rowctr,
                                                             ctx->inlet_reserve, (int)ctx->cap);
    k_inject_count<<<1, 1, 0, st>>>(ctx->d_count, ctx->inlet_rowctr, ctx->inlet_reserve);
    ctx->launches += 2;
    // the next sort covers the rows the inlet may have filled
    ctx->n_alloc = std::min(ctx->cap, ctx->n_alloc + (size_t)ctx->inlet_reserve);
  }
  k_end_step<<<mb, NTHREADS, 0, st>>>(ctx->d_opt, ctx->ts, ctx->nmem);
  ctx->launches += 2;
  ctx->pending_dead = true;
  ctx->has_dead = true;
  if (ctx->rec) {
    dcopy(ctx->rec->bc3, ctx->A.bc, (size_t)n, st);
    dcopy(ctx->rec->ts, ctx->ts, sizeof(TimeState), st);
  }
  record_ev(ctx, 10);
  CK(cudaGetLastError());
  return PLUME_OK;
}

// events of a step: 0 start, 1 after dt, 2 after search and wall boundary,
// 3 after adaptive, 4 after hmax, 5 after momentum, 6 after commit, 7 after
// density, 8 after commit, 9 after velocity, 10 end, 11 before the momentum
// pair sweep, 12 after the position update, 13 after search (before the
// wall boundary).  Phases: 0 search (keys, sort, gather, cell table), 1
// adaptive h, 2 lists, 3 momentum, 4 commit, 5 density, 6 commit, 7 LANS
// filter, 8 position update, 9 dt, 10 total, 11 momentum pair sweep alone,
// 12 inlet (add_new_erupt) and step end, 13 wall boundary (apply_bcond)
static void accumulate_phases(plume_ctx* ctx, const cudaEvent_t* e) {
  float t[NPHASE];
  cudaEventElapsedTime(&t[9], e[0], e[1]);
  cudaEventElapsedTime(&t[0], e[1], e[13]);
  cudaEventElapsedTime(&t[13], e[13], e[2]);
  cudaEventElapsedTime(&t[12], e[12], e[10]);
  cudaEventElapsedTime(&t[1], e[2], e[3]);
  cudaEventElapsedTime(&t[2], e[3], e[4]);
  cudaEventElapsedTime(&t[3], e[4], e[5]);
  cudaEventElapsedTime(&t[4], e[5], e[6]);
  cudaEventElapsedTime(&t[5], e[6], e[7]);
  cudaEventElapsedTime(&t[6], e[7], e[8]);
  cudaEventElapsedTime(&t[7], e[8], e[9]);
  cudaEventElapsedTime(&t[8], e[9], e[12]);
  cudaEventElapsedTime(&t[10], e[0], e[10]);
  cudaEventElapsedTime(&t[11], e[11], e[5]);
  for (int k = 0; k < NPHASE; k++) ctx->phase_ms[k] += t[k];
}

static int ensure_events(plume_ctx* ctx, int nsteps) {
  size_t need = (size_t)NEV * (size_t)(nsteps > 0 ? nsteps : 1);
  while (ctx->evs.size() < need) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    ctx->evs.push_back(e);
  }
  return PLUME_OK;
}

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

const char* plume_version(void) { return "0.1.0"; }

int plume_last_error(plume_ctx* ctx, char* buf, size_t len) {
  if (!buf || !len) return PLUME_E_INVALID;
  const std::string& s = ctx ? ctx->err : g_create_error;
  snprintf(buf, len, "%s", s.c_str());
  return PLUME_OK;
}

// Options every member of an ensemble shares (the sweeps read them once per
// launch); the others (cfl, mixture constants, vent, times, max_steps) are
// per member.
static bool same_shared_options(const PlumeOptions& a, const PlumeOptions& b) {
  return a.dim == b.dim && a.precision == b.precision && a.kernel == b.kernel && a.lans == b.lans &&
         a.energy_smooth == b.energy_smooth && a.pghost_contrib == b.pghost_contrib &&
         a.adaptive_sml == b.adaptive_sml && a.sml_interval == b.sml_interval && a.num_loop == b.num_loop &&
         a.thresh == b.thresh && a.c_smooth == b.c_smooth && a.eta_smooth == b.eta_smooth &&
         a.alpha == b.alpha && a.beta == b.beta && a.ata == b.ata && a.cutoff2 == b.cutoff2 &&
         a.list_factor == b.list_factor && a.g == b.g && a.method == b.method &&
         a.gsph_solver == b.gsph_solver && a.gsph_recon == b.gsph_recon && a.gsph_vol == b.gsph_vol &&
         a.gsph_mono == b.gsph_mono && a.gsph_gradients == b.gsph_gradients &&
         a.gsph_wave_speed == b.gsph_wave_speed;
}

static int create_ctx(const PlumeOptions* opts, const PlumeGrid* grids, int nmem, bool batch, plume_ctx** out) {
  if (!opts || !grids || !out || nmem < 1) {
    g_create_error = "null argument";
    return PLUME_E_INVALID;
  }
  if (nmem > PLUME_MAX_MEMBERS) {
    g_create_error = "too many members";
    return PLUME_E_INVALID;
  }
  const PlumeOptions* opt = &opts[0];
  if (opt->dim != 1 && opt->dim != 3) {
    g_create_error = "dim must be 1 or 3";
    return PLUME_E_INVALID;
  }
  if (opt->method != PLUME_METHOD_SPH && opt->method != PLUME_METHOD_GSPH && opt->method != PLUME_METHOD_GSPH_RCM) {
    g_create_error = "method must be PLUME_METHOD_SPH, PLUME_METHOD_GSPH or PLUME_METHOD_GSPH_RCM";
    return PLUME_E_INVALID;
  }
  if (opt->method != PLUME_METHOD_SPH) {
    const int r = opt->gsph_recon;
    const int sv = opt->gsph_solver;
    if (!(sv == PLUME_RIEMANN_ROE || sv == PLUME_RIEMANN_HLLC || sv == PLUME_RIEMANN_HLLC_MY ||
          sv == PLUME_RIEMANN_VANLEER) ||
        !(r == 0 || r == 1 || r == 2 || r == 3 || r == 4 || r == 10) ||
        !(opt->gsph_vol == 0 || opt->gsph_vol == 1 || opt->gsph_vol == 3) ||
        (opt->gsph_mono != 0 && opt->gsph_mono != 1) ||
        (sv == PLUME_RIEMANN_HLLC_MY && opt->gsph_wave_speed != 2 && opt->gsph_wave_speed != 3)) {
      g_create_error = "GSPH: solver ROE/HLLC/HLLC_MY/VANLEER (HLLC_MY with wave speed 2 or 3), recon 0-4 or 10, "
                       "vol 0, 1 or 3, mono 0 or 1";
      return PLUME_E_INVALID;
    }
  }
  size_t capacity = 0;
  double ncell_tot = 0, nbk_tot = 0;
  for (int m = 0; m < nmem; m++) {
    const PlumeOptions& om = opts[m];
    const PlumeGrid& gm = grids[m];
    if (m > 0 && !same_shared_options(om, *opt)) {
      g_create_error = "member " + std::to_string(m) + ": options differ from member 0 in a shared field";
      return PLUME_E_INVALID;
    }
    if (om.capacity == 0) {
      g_create_error = "capacity must be >= 1";
      return PLUME_E_INVALID;
    }
    capacity += om.capacity;
    if (gm.del <= 0 || gm.nb[0] < 1 || gm.nb[1] < 1 || gm.nb[2] < 1 ||
        (opt->dim == 1 && (gm.nb[1] != 1 || gm.nb[2] != 1))) {
      g_create_error = "invalid bucket grid" + (nmem > 1 ? " of member " + std::to_string(m) : std::string());
      return PLUME_E_INVALID;
    }
    const int s = gm.subcells > 0 ? gm.subcells : 1;
    ncell_tot += (double)gm.nb[0] * s * (opt->dim == 3 ? (double)gm.nb[1] * s * gm.nb[2] * s : 1.0);
    nbk_tot += (opt->dim == 3) ? (double)gm.nb[0] * gm.nb[1] * gm.nb[2] : 1.0;
  }
  if (capacity > (size_t)0x7fffffff) {
    g_create_error = "capacity must be in [1, 2^31)";
    return PLUME_E_INVALID;
  }
  if (ncell_tot > 2.0e9 || nbk_tot > 2.0e9) {
    g_create_error = "too many fine cells";
    return PLUME_E_INVALID;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    g_create_error = "no CUDA device";
    return PLUME_E_CUDA;
  }
  plume_ctx* ctx = new plume_ctx();
  ctx->opt = *opt;
  ctx->o = make_opt(*opt);
  ctx->nmem = nmem;
  ctx->batch = batch;
  ctx->hgeo.resize(nmem);
  ctx->hopt.resize(nmem);
  uint32_t cell_base = 0;
  int bucket_base = 0;
  std::vector<uint16_t> bmember;
  for (int m = 0; m < nmem; m++) {
    const PlumeGrid* grid = &grids[m];
    const int s = grid->subcells > 0 ? grid->subcells : 1;
    Geo& g = ctx->hgeo[m];
    g = Geo{};
    for (int a = 0; a < 3; a++) {
      g.mind[a] = grid->mindom[a];
      g.nb[a] = grid->nb[a];
      g.lo[a] = grid->domain_lo[a];
      g.hi[a] = grid->domain_hi[a];
    }
    g.del = grid->del;
    g.s = s;
    g.cw = grid->del / s;
    g.idel = 1.0 / g.del;
    g.icw = 1.0 / g.cw;
    g.icwf = (float)g.icw;
    g.dim = opt->dim;
    for (int a = 0; a < 3; a++) g.G[a] = (opt->dim == 3 || a == 0) ? g.nb[a] * s : 1;
    g.nbk = (opt->dim == 3) ? g.nb[0] * g.nb[1] * g.nb[2] : 1;
    g.cell_base = cell_base;
    g.bucket_base = bucket_base;
    cell_base += (uint32_t)((size_t)g.G[0] * g.G[1] * g.G[2]);
    bucket_base += g.nbk;
    bmember.insert(bmember.end(), (size_t)g.nbk, (uint16_t)m);
    ctx->hopt[m] = make_opt(opts[m]);
  }
  ctx->ncells = cell_base;
  ctx->keybits = 1;
  while ((1ull << ctx->keybits) <= (unsigned long long)ctx->ncells) ctx->keybits++;
  ctx->nbk = bucket_base;
  ctx->cap = capacity;
  ctx->sweep_warp = (opt->precision == PLUME_PREC_FP64);
  if (const char* sw = getenv("PLUME_SWEEP")) {
    if (!strcmp(sw, "warp")) { ctx->sweep_warp = true; ctx->use_lists = false; }
    if (!strcmp(sw, "thread")) { ctx->sweep_warp = false; ctx->use_lists = false; }
    if (!strcmp(sw, "list")) { ctx->sweep_warp = false; ctx->use_lists = true; }
    if (!strcmp(sw, "list_warp")) { ctx->sweep_warp = false; ctx->use_lists = true; ctx->list_warp = true; }
  }
  if (opt->dim == 3 && ctx->use_lists && capacity > (size_t)NL_JMASK) {
    g_create_error = "capacity above the neighbour-list index range (2^26)";
    delete ctx;
    return PLUME_E_INVALID;
  }
  int rc = PLUME_OK;
  auto fail = [&](int code) {
    g_create_error = ctx->err;
    plume_destroy(ctx);
    return code;
  };
  if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess) {
    ctx->err = "cudaStreamCreate failed";
    return fail(PLUME_E_CUDA);
  }
  if ((rc = ensure_events(ctx, 1))) return fail(rc);
  ctx->ev = ctx->evs.data();
  if ((rc = alloc_dev(ctx, ctx->A, ctx->cap)) || (rc = alloc_dev(ctx, ctx->B, ctx->cap))) return fail(rc);
  {
    size_t c = ctx->cap;
    double** w[] = {&ctx->W.hlist, &ctx->W.nv0, &ctx->W.nv1, &ctx->W.nv2, &ctx->W.ne, &ctx->W.nrho,
                    &ctx->W.nY, &ctx->W.nE};
    for (auto p : w)
      if ((rc = dev_alloc(ctx, (void**)p, 8 * c))) return fail(rc);
    if ((rc = dev_alloc(ctx, (void**)&ctx->W.xr, 4 * c)) || (rc = dev_alloc(ctx, (void**)&ctx->W.yr, 4 * c)) ||
        (rc = dev_alloc(ctx, (void**)&ctx->W.zr, 4 * c)))
      return fail(rc);
    if (opt->dim == 3 && ctx->use_lists) {
      if ((rc = dev_alloc(ctx, (void**)&ctx->L.e, sizeof(uint2) * (size_t)LCAP * c)) ||
          (rc = dev_alloc(ctx, (void**)&ctx->L.cnt, sizeof(uint16_t) * c)) ||
          (rc = dev_alloc(ctx, (void**)&ctx->rflag, 4 * c)) ||
          (rc = dev_alloc(ctx, (void**)&ctx->roffs, 8 * c)) ||
          (rc = dev_alloc(ctx, (void**)&ctx->rsums, 8 * (c / 1024 + 2))) ||
          (rc = dev_alloc(ctx, (void**)&ctx->rtot, 8)) ||
          (rc = dev_alloc(ctx, (void**)&ctx->real_idx, 4 * c)) ||
          (rc = dev_alloc(ctx, (void**)&ctx->d_real, sizeof(int))))
        return fail(rc);
      const char* tl = getenv("PLUME_TILES");
      if (nmem == 1 && !(tl && !strcmp(tl, "0"))) {
        const Geo& g0 = ctx->hgeo[0];
        const long long nt = (long long)((g0.G[0] + TILE_X - 1) / TILE_X) * ((g0.G[1] + TILE_Y - 1) / TILE_Y) *
                             ((g0.G[2] + TILE_Z - 1) / TILE_Z);
        if (nt > 0 && nt < (1ll << 30)) {
          ctx->ntiles = (int)nt;
          if ((rc = dev_alloc(ctx, (void**)&ctx->tcount, 4 * (size_t)nt)) ||
              (rc = dev_alloc(ctx, (void**)&ctx->toffs, 8 * (size_t)nt)) ||
              (rc = dev_alloc(ctx, (void**)&ctx->tsums, 8 * ((size_t)nt / 1024 + 2))) ||
              (rc = dev_alloc(ctx, (void**)&ctx->ttot, 8)) ||
              (rc = dev_alloc(ctx, (void**)&ctx->real_tile, 4 * c)) ||
              (rc = dev_alloc(ctx, (void**)&ctx->d_real_tile, sizeof(int))))
            return fail(rc);
        }
      }
    }
    if (opt->method != PLUME_METHOD_SPH &&
        (rc = dev_alloc(ctx, (void**)&ctx->grad, 8 * c * (size_t)((opt->dim + 2) * opt->dim))))
      return fail(rc);
    if (opt->precision == PLUME_PREC_MIXED && opt->dim == 3) {
      if ((rc = dev_alloc(ctx, (void**)&ctx->K.P, 16 * c)) || (rc = dev_alloc(ctx, (void**)&ctx->K.Q, 16 * c)) ||
          (rc = dev_alloc(ctx, (void**)&ctx->K.R, 16 * c)) || (rc = dev_alloc(ctx, (void**)&ctx->K.S, 16 * c)))
        return fail(rc);
    }
    if ((rc = dev_alloc(ctx, (void**)&ctx->keys, 4 * c)) || (rc = dev_alloc(ctx, (void**)&ctx->perm, 4 * c)) ||
        (rc = dev_alloc(ctx, (void**)&ctx->cs, 4 * ((size_t)ctx->ncells + 2))) ||
        (rc = dev_alloc(ctx, (void**)&ctx->d_count, sizeof(int))) ||
        (rc = dev_alloc(ctx, (void**)&ctx->ts, sizeof(TimeState) * (size_t)nmem)) ||
        (rc = dev_alloc(ctx, (void**)&ctx->hb, 8 * (size_t)ctx->nbk)) ||
        (rc = dev_alloc(ctx, (void**)&ctx->h27, 8 * (size_t)ctx->nbk)) ||
        (rc = dev_alloc(ctx, (void**)&ctx->d_geo, sizeof(Geo) * (size_t)nmem)) ||
        (rc = dev_alloc(ctx, (void**)&ctx->d_opt, sizeof(Opt) * (size_t)nmem)) ||
        (rc = dev_alloc(ctx, (void**)&ctx->bmember, 2 * (size_t)ctx->nbk)) ||
        (rc = dev_alloc(ctx, (void**)&ctx->d_hstep, sizeof(int))))
      return fail(rc);
    if (ctx->sorter.reserve((int)c) != cudaSuccess) {
      ctx->err = "radix sort buffers";
      return fail(PLUME_E_CUDA);
    }
  }
  bool any_flags = false, any_face = false;
  for (int m = 0; m < nmem; m++) {
    any_flags |= grids[m].flags != nullptr;
    any_face |= grids[m].face_index != nullptr;
  }
  if (opt->dim == 3 && any_flags) {
    std::vector<uint8_t> f((size_t)ctx->nbk, 0);
    for (int m = 0; m < nmem; m++)
      if (grids[m].flags) memcpy(f.data() + ctx->hgeo[m].bucket_base, grids[m].flags, ctx->hgeo[m].nbk);
    if ((rc = dev_alloc(ctx, (void**)&ctx->bflags, ctx->nbk))) return fail(rc);
    cudaMemcpy(ctx->bflags, f.data(), ctx->nbk, cudaMemcpyHostToDevice);
  }
  if (opt->dim == 3 && any_face) {
    std::vector<int8_t> f(6 * (size_t)ctx->nbk, 0);
    for (int m = 0; m < nmem; m++)
      if (grids[m].face_index)
        memcpy(f.data() + 6 * (size_t)ctx->hgeo[m].bucket_base, grids[m].face_index, 6 * (size_t)ctx->hgeo[m].nbk);
    if ((rc = dev_alloc(ctx, (void**)&ctx->bface, 6 * (size_t)ctx->nbk))) return fail(rc);
    cudaMemcpy(ctx->bface, f.data(), 6 * (size_t)ctx->nbk, cudaMemcpyHostToDevice);
  }
  if (opt->dim == 3) {
    // involvement: NONE where absorbing, POTENTIAL elsewhere (dataread.cc:457)
    std::vector<uint8_t> st((size_t)ctx->nbk, PLUME_BINV_POTENTIAL);
    for (int m = 0; m < nmem; m++)
      if (grids[m].flags)
        for (int b = 0; b < ctx->hgeo[m].nbk; b++) {
          const uint8_t f = grids[m].flags[b];
          if (f & PLUME_BUCKET_ABSORBING) st[ctx->hgeo[m].bucket_base + b] = PLUME_BINV_NONE;
          if (f & (PLUME_BUCKET_UNDERGROUND | PLUME_BUCKET_PRESS_BC)) ctx->explicit_types = 1;
        }
    if ((rc = dev_alloc(ctx, (void**)&ctx->binv, ctx->nbk)) ||
        (rc = dev_alloc(ctx, (void**)&ctx->bmark, ctx->nbk)) ||
        (rc = dev_alloc(ctx, (void**)&ctx->d_adapt, sizeof(int) * (size_t)nmem)))
      return fail(rc);
    cudaMemcpy(ctx->binv, st.data(), ctx->nbk, cudaMemcpyHostToDevice);
  }
  if (cudaMallocHost(&ctx->h_ts, sizeof(TimeState) * (size_t)nmem) != cudaSuccess) {
    ctx->err = "cudaMallocHost";
    return fail(PLUME_E_CUDA);
  }
  for (int m = 0; m < nmem; m++) {
    TimeState t{};
    t.time = 0;
    t.ndtimeoutput = opts[m].timeoutput;
    t.dtmin_bits = 0;
    t.active = 1;
    t.freeze = batch ? 1 : 0;
    ctx->h_ts[m] = t;
  }
  int zero = 0;
  if (cudaMemcpy(ctx->ts, ctx->h_ts, sizeof(TimeState) * (size_t)nmem, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->d_geo, ctx->hgeo.data(), sizeof(Geo) * (size_t)nmem, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->d_opt, ctx->hopt.data(), sizeof(Opt) * (size_t)nmem, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->bmember, bmember.data(), 2 * (size_t)ctx->nbk, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->d_hstep, &zero, sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->d_count, &zero, sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
    ctx->err = "init member tables";
    return fail(PLUME_E_CUDA);
  }
  if (cudaDeviceSynchronize() != cudaSuccess) {
    ctx->err = "device init";
    return fail(PLUME_E_CUDA);
  }
  *out = ctx;
  return PLUME_OK;
}

int plume_create(const PlumeOptions* opt, const PlumeGrid* grid, plume_ctx** out) {
  return create_ctx(opt, grid, 1, false, out);
}

int plume_batch_create(const PlumeOptions* opts, const PlumeGrid* grids, int nmembers, plume_ctx** out) {
  return create_ctx(opts, grids, nmembers, true, out);
}

int plume_destroy(plume_ctx* ctx) {
  if (!ctx) return PLUME_OK;
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
  if (ctx->img_key) cudaFree(ctx->img_key);
  if (ctx->img_xyz) cudaFree(ctx->img_xyz);
  if (ctx->bc_map) cudaFree(ctx->bc_map);
  if (ctx->d_nreal) cudaFree(ctx->d_nreal);
  if (ctx->snap_st) cudaStreamSynchronize(ctx->snap_st);
  {  // staging arrays (null when never allocated)
    void* sp[] = {ctx->snap.key, ctx->snap.x, ctx->snap.y, ctx->snap.z, ctx->snap.vx, ctx->snap.vy, ctx->snap.vz,
                  ctx->snap.mass, ctx->snap.h, ctx->snap.rho, ctx->snap.e, ctx->snap.p, ctx->snap.Y,
                  ctx->snap.phase, ctx->snap.bc, ctx->snap.inv};
    for (void* q : sp) if (q) cudaFree(q);
  }
  if (ctx->snap_staged) cudaEventDestroy(ctx->snap_staged);
  if (ctx->snap_done) cudaEventDestroy(ctx->snap_done);
  if (ctx->snap_st) cudaStreamDestroy(ctx->snap_st);
  if (ctx->snap_ts) cudaFreeHost(ctx->snap_ts);
  if (ctx->inlet_buf) cudaFree(ctx->inlet_buf);
  if (ctx->inlet_colcnt) cudaFree(ctx->inlet_colcnt);
  if (ctx->inlet_rowctr) cudaFree(ctx->inlet_rowctr);
  for (void* p : ctx->adj_allocs) cudaFree(p);
  for (auto e : ctx->run_ev)
    if (e) cudaEventDestroy(e);
  for (void* p : ctx->allocs) cudaFree(p);
  ctx->sorter.release();
  if (ctx->h_ts) cudaFreeHost(ctx->h_ts);
  for (auto& e : ctx->evs)
    if (e) cudaEventDestroy(e);
  if (ctx->st) cudaStreamDestroy(ctx->st);
  delete ctx;
  return PLUME_OK;
}

// ---- host <-> device particle copies
// A table of copies in one launch: when every host array is page-locked
// (mapped into the device's address space), the device moves the whole
// particle table itself, reading or writing host memory over the
// CPU-GPU link, instead of one DMA transfer per field.
struct CopyJob {
  char* dst;
  const char* src;
  unsigned long long bytes;
};
struct CopyJobs {
  CopyJob j[24];
  int n;
};
__global__ void k_copy_multi(CopyJobs J) {
  const CopyJob c = J.j[blockIdx.y];
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const uintptr_t al = (uintptr_t)c.dst | (uintptr_t)c.src;
  size_t done = 0;
  if ((al & 15) == 0) {
    const size_t nv = c.bytes >> 4;
    const uint4* sv = reinterpret_cast<const uint4*>(c.src);
    uint4* dv = reinterpret_cast<uint4*>(c.dst);
    for (size_t k = tid; k < nv; k += stride) dv[k] = sv[k];
    done = nv << 4;
  } else if ((al & 7) == 0) {
    const size_t nv = c.bytes >> 3;
    const uint2* sv = reinterpret_cast<const uint2*>(c.src);
    uint2* dv = reinterpret_cast<uint2*>(c.dst);
    for (size_t k = tid; k < nv; k += stride) dv[k] = sv[k];
    done = nv << 3;
  }
  for (size_t k = done + tid; k < c.bytes; k += stride) c.dst[k] = c.src[k];
}

// device-side address of a page-locked host array, or null
static void* mapped_host(const void* h) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// issues the copies (the host side is src for H2D, dst for D2H); one kernel
// when every host array is mapped, else one cudaMemcpyAsync each (also for
// device-to-device copies)
static int run_copies(plume_ctx* ctx, const std::vector<CopyJob>& jobs, cudaMemcpyKind kind) {
  cudaStream_t st = ctx->st;
  const bool h2d = kind == cudaMemcpyHostToDevice;
  CopyJobs J{};
  bool mapped = jobs.size() <= 24 && (h2d || kind == cudaMemcpyDeviceToHost);
  for (size_t q = 0; q < jobs.size() && mapped; q++) {
    CopyJob c = jobs[q];
    void* dp = mapped_host(h2d ? (const void*)c.src : (const void*)c.dst);
    if (!dp) {
      mapped = false;
      break;
    }
    if (h2d) c.src = (const char*)dp; else c.dst = (char*)dp;
    J.j[J.n++] = c;
  }
  if (mapped && J.n > 0) {
    dim3 grid(2 * 152, J.n);
    k_copy_multi<<<grid, 256, 0, st>>>(J);
    ctx->launches++;
    CK(cudaGetLastError());
    return PLUME_OK;
  }
  for (const CopyJob& c : jobs)
    if (c.bytes) CK(cudaMemcpyAsync(c.dst, c.src, c.bytes, kind, st));
  return PLUME_OK;
}

static int check_soa(plume_ctx* ctx, const PlumeSoA* s) {
  if (!s || !s->key || !s->x || !s->vx || !s->mass || !s->h || !s->rho || !s->e || !s->p || !s->Y ||
      !s->gamma || !s->c || !s->T || !s->cp || !s->phase || !s->bc_type || !s->involved) {
    ctx->err = "missing particle array";
    return PLUME_E_INVALID;
  }
  if (ctx->o.dim == 3 && (!s->y || !s->z || !s->vy || !s->vz)) {
    ctx->err = "3D particles need y, z, vy, vz";
    return PLUME_E_INVALID;
  }
  return PLUME_OK;
}

// member ids: null = member 0 for every row (single runs)
static int copy_soa(plume_ctx* ctx, const PlumeSoA* s, size_t off, size_t n, cudaMemcpyKind kind,
                    const uint16_t* member = nullptr) {
  int rc = check_soa(ctx, s);
  if (rc) return rc;
  if (member && kind == cudaMemcpyHostToDevice) {
    for (size_t r = 0; r < n; r++)
      if (member[r] >= ctx->nmem) {
        ctx->err = "member id out of range at row " + std::to_string(r);
        return PLUME_E_INVALID;
      }
  }
  const bool d3 = ctx->o.dim == 3;
  cudaStream_t st = ctx->st;
  Dev& A = ctx->A;
  std::vector<CopyJob> jobs;
  auto job = [&](void* d, const void* h, size_t bytes) { jobs.push_back(CopyJob{(char*)d, (const char*)h, bytes}); };
  job(A.key + off, s->key, 8 * n);
  struct F { double* d; const double* h; } f[] = {
      {A.x, s->x}, {A.vx, s->vx}, {A.mass, s->mass}, {A.h, s->h}, {A.rho, s->rho}, {A.e, s->e},
      {A.p, s->p}, {A.Y, s->Y}, {A.gam, s->gamma}, {A.c, s->c}, {A.T, s->T}, {A.cp, s->cp}};
  for (auto& q : f) job(q.d + off, q.h, 8 * n);
  if (d3) {
    job(A.y + off, s->y, 8 * n);
    job(A.z + off, s->z, 8 * n);
    job(A.vy + off, s->vy, 8 * n);
    job(A.vz + off, s->vz, 8 * n);
  }
  // smoothed velocity: optional on upload (zero when absent)
  double* vs[3] = {A.vsx, A.vsy, A.vsz};
  const double* hv[3] = {s->vsx, s->vsy, s->vsz};
  for (int a = 0; a < (d3 ? 3 : 1); a++) {
    if (hv[a])
      job(vs[a] + off, hv[a], 8 * n);
    else
      CK(cudaMemsetAsync(vs[a] + off, 0, 8 * n, st));
  }
  job(A.phase + off, s->phase, n);
  job(A.bc + off, s->bc_type, n);
  job(A.inv + off, s->involved, n);
  if (member)
    job(A.mem + off, member, 2 * n);
  else
    CK(cudaMemsetAsync(A.mem + off, 0, 2 * n, st));
  return run_copies(ctx, jobs, kind);
}

static int set_count(plume_ctx* ctx, size_t n) {
  ctx->n_alloc = n;
  int v = (int)n;
  CK(cudaMemcpyAsync(ctx->d_count, &v, sizeof(int), cudaMemcpyHostToDevice, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return PLUME_OK;
}

int plume_upload(plume_ctx* ctx, const PlumeSoA* host, size_t n) {
  if (!ctx) return PLUME_E_INVALID;
  if (n > ctx->cap) {
    ctx->err = "particle count exceeds capacity";
    return PLUME_E_CAPACITY;
  }
  int rc = copy_soa(ctx, host, 0, n, cudaMemcpyHostToDevice);
  if (rc) return rc;
  rc = set_count(ctx, n);
  if (rc) return rc;
  ctx->pending_dead = true;  // order unknown: search before any pair query
  return PLUME_OK;
}

int plume_upload_device(plume_ctx* ctx, const PlumeSoA* dev, size_t n) {
  if (!ctx) return PLUME_E_INVALID;
  if (n > ctx->cap) {
    ctx->err = "particle count exceeds capacity";
    return PLUME_E_CAPACITY;
  }
  int rc = copy_soa(ctx, dev, 0, n, cudaMemcpyDeviceToDevice);
  if (rc) return rc;
  rc = set_count(ctx, n);
  if (rc) return rc;
  ctx->pending_dead = true;
  return PLUME_OK;
}

int plume_append(plume_ctx* ctx, const PlumeSoA* host, size_t n) {
  if (!ctx) return PLUME_E_INVALID;
  if (ctx->n_alloc + n > ctx->cap) {
    ctx->err = "append exceeds capacity";
    return PLUME_E_CAPACITY;
  }
  int rc = copy_soa(ctx, host, ctx->n_alloc, n, cudaMemcpyHostToDevice);
  if (rc) return rc;
  rc = set_count(ctx, ctx->n_alloc + n);
  ctx->pending_dead = true;
  return rc;
}

int plume_set_ghost_state(plume_ctx* ctx, const uint64_t* keys, const double* state, const double* Y, size_t n) {
  if (!ctx || (n && (!keys || !state))) return PLUME_E_INVALID;
  if (n == 0) return PLUME_OK;
  const int w = ctx->o.dim + 2;
  std::vector<size_t> ord(n);
  for (size_t i = 0; i < n; i++) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return keys[a] < keys[b]; });
  std::vector<uint64_t> k(n);
  std::vector<double> s(n * w), y(Y ? n : 0);
  for (size_t r = 0; r < n; r++) {
    k[r] = keys[ord[r]];
    for (int c = 0; c < w; c++) s[r * w + c] = state[ord[r] * w + c];
    if (Y) y[r] = Y[ord[r]];
  }
  uint64_t* dk = nullptr;
  double *ds = nullptr, *dy = nullptr;
  CK(cudaMalloc(&dk, 8 * n));
  CK(cudaMalloc(&ds, 8 * n * w));
  if (Y) CK(cudaMalloc(&dy, 8 * n));
  CK(cudaMemcpy(dk, k.data(), 8 * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ds, s.data(), 8 * n * w, cudaMemcpyHostToDevice));
  if (Y) CK(cudaMemcpy(dy, y.data(), 8 * n, cudaMemcpyHostToDevice));
  k_set_ghost<<<nblocks(ctx->n_alloc ? ctx->n_alloc : 1), NTHREADS, 0, ctx->st>>>(
      ctx->d_opt, ctx->A, ctx->d_count, dk, ds, dy, (int)n, ctx->o.dim);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->st));
  cudaFree(dk);
  cudaFree(ds);
  if (dy) cudaFree(dy);
  return PLUME_OK;
}

static int finish_steps(plume_ctx* ctx) {
  int s = ctx_sync_status(ctx);
  int n = 0;
  CK(cudaMemcpy(&n, ctx->d_count, sizeof(int), cudaMemcpyDeviceToHost));
  ctx->n_alloc = (size_t)n;
  return s;
}

int plume_steps(plume_ctx* ctx, int nsteps, PlumeStepLog* log) {
  if (!ctx || nsteps < 0) return PLUME_E_INVALID;
  for (auto& v : ctx->phase_ms) v = 0;
  ctx->launches = 0;
  int rc0 = ensure_events(ctx, nsteps);
  if (rc0) return rc0;
  for (int k = 0; k < nsteps; k++) {
    ctx->ev = ctx->evs.data() + (size_t)NEV * k;
    int rc = step_async(ctx);
    if (rc) return rc;
    if (log) {
      int s = finish_steps(ctx);
      accumulate_phases(ctx, ctx->ev);
      // the particle count shrinks only at the next search
      PlumeStepLog& L = log[k];
      L.dt = ctx->h_ts[0].dtime;
      L.time = ctx->h_ts[0].time;
      L.step = ctx->h_ts[0].step;
      L.status = s;
      L.n_total = ctx->n_alloc;
      L.n_real = 0;
      L.n_lost = 0;
      for (int m = 0; m < ctx->nmem; m++) {
        L.n_real += ctx->h_ts[m].n_real;
        L.n_lost += ctx->h_ts[m].n_lost;
      }
      if (s) return s;
    }
  }
  int s = finish_steps(ctx);
  if (!log)
    for (int k = 0; k < nsteps; k++) accumulate_phases(ctx, ctx->evs.data() + (size_t)NEV * k);
  return s;
}

int plume_step(plume_ctx* ctx, double* dt_out) {
  int rc = plume_steps(ctx, 1, nullptr);
  if (dt_out && ctx) *dt_out = ctx->h_ts->dtime;
  return rc;
}

int plume_adapt_sml(plume_ctx* ctx) {
  if (!ctx) return PLUME_E_INVALID;
  int rc = search(ctx);
  if (rc) return rc;
  const int nb = nblocks(ctx->n_alloc ? ctx->n_alloc : 1);
  const bool mixed = ctx->opt.precision == PLUME_PREC_MIXED;
  if (ctx->o.dim == 3) {
    if (mixed) k_adaptive<3, float><<<nb, NTHREADS, 0, ctx->st>>>(ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->d_count, ctx->ts, ctx->d_hstep, 1);
    else k_adaptive<3, double><<<nb, NTHREADS, 0, ctx->st>>>(ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->d_count, ctx->ts, ctx->d_hstep, 1);
  } else {
    if (mixed) k_adaptive<1, float><<<nb, NTHREADS, 0, ctx->st>>>(ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->d_count, ctx->ts, ctx->d_hstep, 1);
    else k_adaptive<1, double><<<nb, NTHREADS, 0, ctx->st>>>(ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->d_count, ctx->ts, ctx->d_hstep, 1);
  }
  CK(cudaGetLastError());
  return ctx_sync_status(ctx);
}

// real particles (bc 100 or 99) of [0, count): one atomic per warp
__global__ void k_count_real(Dev A, const int* __restrict__ d_count, int n, unsigned long long* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool r = i < n && i < *d_count && is_real(A.bc[i]);
  const unsigned b = __ballot_sync(0xffffffffu, r);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(out, (unsigned long long)__popc(b));
}

// live rows (not deleted) of [0, count)
__global__ void k_live_flags(Dev A, const int* __restrict__ d_count, int n, unsigned int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  flag[i] = (i < *d_count && A.bc[i] != BC_DEAD) ? 1u : 0u;
}
__global__ void k_live_scatter(const unsigned int* __restrict__ flag, const unsigned long long* __restrict__ offs,
                               int n, uint32_t* __restrict__ perm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flag[i]) perm[offs[i]] = (uint32_t)i;
}

// drops the rows deleted by the last steps without re-sorting (the next
// step sorts anyway); a search where the scan buffers are absent
static int compact(plume_ctx* ctx) {
  if (!ctx->rflag) return search(ctx);
  cudaStream_t st = ctx->st;
  const int n = (int)ctx->n_alloc;
  if (n > 0) {
    const int nsb = (n + 1023) / 1024;
    k_live_flags<<<nblocks(n), NTHREADS, 0, st>>>(ctx->A, ctx->d_count, n, ctx->rflag);
    k_scan_blocks<<<nsb, 1024, 0, st>>>(ctx->rflag, n, ctx->roffs, ctx->rsums);
    k_scan_sums<<<1, 1024, 0, st>>>(ctx->rsums, nsb, ctx->rtot);
    k_scan_add<<<nsb, 1024, 0, st>>>(ctx->roffs, n, ctx->rsums);
    k_live_scatter<<<nblocks(n), NTHREADS, 0, st>>>(ctx->rflag, ctx->roffs, n, ctx->perm);
    unsigned long long live = 0;
    CK(cudaMemcpyAsync(&live, ctx->rtot, sizeof(live), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (live) k_gather<<<nblocks((size_t)live), NTHREADS, 0, st>>>(ctx->d_geo, ctx->A, ctx->B, ctx->W, ctx->perm, (int)live);
    std::swap(ctx->A, ctx->B);
    const int nl = (int)live;
    CK(cudaMemcpyAsync(ctx->d_count, &nl, sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    ctx->n_alloc = live;
  }
  ctx->has_dead = false;
  return PLUME_OK;
}

int plume_count(plume_ctx* ctx, size_t* n_total, size_t* n_real) {
  if (!ctx) return PLUME_E_INVALID;
  if (ctx->has_dead) {
    int rc = compact(ctx);
    if (rc) return rc;
    int s = ctx_sync_status(ctx);
    if (s) return s;
    int n = 0;
    CK(cudaMemcpy(&n, ctx->d_count, sizeof(int), cudaMemcpyDeviceToHost));
    ctx->n_alloc = (size_t)n;
  }
  if (n_total) *n_total = ctx->n_alloc;
  if (n_real) {
    if (!ctx->d_nreal) CK(cudaMalloc(&ctx->d_nreal, sizeof(unsigned long long)));
    CK(cudaMemsetAsync(ctx->d_nreal, 0, sizeof(unsigned long long), ctx->st));
    const int n = (int)ctx->n_alloc;
    if (n) k_count_real<<<nblocks(n), NTHREADS, 0, ctx->st>>>(ctx->A, ctx->d_count, n, ctx->d_nreal);
    unsigned long long r = 0;
    CK(cudaMemcpyAsync(&r, ctx->d_nreal, sizeof(r), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    *n_real = (size_t)r;
  }
  return PLUME_OK;
}

int plume_download(plume_ctx* ctx, PlumeSoA* host, size_t cap, size_t* n) {
  if (!ctx || !host || !n) return PLUME_E_INVALID;
  size_t nt = 0;
  int rc = plume_count(ctx, &nt, nullptr);
  if (rc) return rc;
  *n = nt;
  if (nt > cap) {
    ctx->err = "download capacity too small";
    return PLUME_E_CAPACITY;
  }
  rc = check_soa(ctx, host);
  if (rc) return rc;
  Dev& A = ctx->A;
  cudaStream_t st = ctx->st;
  std::vector<CopyJob> jobs;
  auto d2h = [&](void* h, const void* d, size_t bytes) {
    if (h) jobs.push_back(CopyJob{(char*)h, (const char*)d, bytes});
  };
  d2h(host->key, A.key, 8 * nt);
  const double* src[] = {A.x, A.y, A.z, A.vx, A.vy, A.vz, A.vsx, A.vsy, A.vsz, A.mass, A.h, A.rho, A.e,
                         A.p, A.Y, A.gam, A.c, A.T, A.cp};
  double* dst[] = {host->x, host->y, host->z, host->vx, host->vy, host->vz, host->vsx, host->vsy,
                   host->vsz, host->mass, host->h, host->rho, host->e, host->p, host->Y, host->gamma,
                   host->c, host->T, host->cp};
  const bool d3 = ctx->o.dim == 3;
  for (int f = 0; f < 19; f++) {
    bool axis = (f == 1 || f == 2 || f == 4 || f == 5 || f == 7 || f == 8);
    if (axis && !d3) {
      if (dst[f]) memset(dst[f], 0, 8 * nt);
      continue;
    }
    d2h(dst[f], src[f], 8 * nt);
  }
  d2h(host->phase, A.phase, nt);
  d2h(host->bc_type, A.bc, nt);
  d2h(host->involved, A.inv, nt);
  rc = run_copies(ctx, jobs, cudaMemcpyDeviceToHost);
  if (rc) return rc;
  CK(cudaStreamSynchronize(st));
  return PLUME_OK;
}

int plume_get_time(plume_ctx* ctx, double* time, int* step, int* ioutput) {
  if (!ctx) return PLUME_E_INVALID;
  CK(cudaStreamSynchronize(ctx->st));
  CK(cudaMemcpy(ctx->h_ts, ctx->ts, sizeof(TimeState) * ctx->nmem, cudaMemcpyDeviceToHost));
  if (time) *time = ctx->h_ts->time;
  if (step) *step = ctx->h_ts->step;
  if (ioutput) *ioutput = ctx->h_ts->ioutput;
  return PLUME_OK;
}

int plume_set_time(plume_ctx* ctx, double time, int step, int ioutput, double next_output) {
  if (!ctx) return PLUME_E_INVALID;
  CK(cudaStreamSynchronize(ctx->st));
  CK(cudaMemcpy(ctx->h_ts, ctx->ts, sizeof(TimeState) * ctx->nmem, cudaMemcpyDeviceToHost));
  for (int m = 0; m < ctx->nmem; m++) {  // every member of an ensemble
    ctx->h_ts[m].time = time;
    ctx->h_ts[m].step = step;
    ctx->h_ts[m].ioutput = ioutput;
    ctx->h_ts[m].ndtimeoutput = next_output;
  }
  CK(cudaMemcpy(ctx->ts, ctx->h_ts, sizeof(TimeState) * ctx->nmem, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_hstep, &step, sizeof(int), cudaMemcpyHostToDevice));
  ctx->host_step = step;
  return PLUME_OK;
}

static int neighbor_pairs(plume_ctx* ctx, int mode, const uint64_t* keys, size_t nkeys, uint64_t* key_i,
                          uint64_t* key_j, size_t cap, size_t* n) {
  if (!ctx || !n || (mode != 0 && mode != 1) || (nkeys && !keys) || nkeys > (size_t)INT_MAX)
    return PLUME_E_INVALID;
  ScratchFree subs;
  uint64_t* dsub = nullptr;
  if (keys) {
    std::vector<uint64_t> sk(keys, keys + nkeys);
    std::sort(sk.begin(), sk.end());
    CK(cudaMalloc(&dsub, 8 * (sk.size() ? sk.size() : 1)));
    subs.p[0] = dsub;
    if (!sk.empty()) CK(cudaMemcpy(dsub, sk.data(), 8 * sk.size(), cudaMemcpyHostToDevice));
  }
  const int nsub = (int)nkeys;
  int rc = search(ctx);
  if (rc) return rc;
  int s = ctx_sync_status(ctx);
  if (s) return s;
  int cnt_h = 0;
  CK(cudaMemcpy(&cnt_h, ctx->d_count, sizeof(int), cudaMemcpyDeviceToHost));
  ctx->n_alloc = (size_t)cnt_h;
  const int np = cnt_h;
  unsigned int* cnt = nullptr;
  unsigned long long *offs = nullptr, *sums = nullptr, *tot = nullptr;
  int nbk = (np + 1023) / 1024;
  CK(cudaMalloc(&cnt, 4 * (size_t)(np ? np : 1)));
  CK(cudaMalloc(&offs, 8 * (size_t)(np ? np : 1)));
  CK(cudaMalloc(&sums, 8 * (size_t)(nbk ? nbk : 1)));
  CK(cudaMalloc(&tot, 8));
  cudaStream_t st = ctx->st;
  const int nb = nblocks(np ? np : 1);
  if (ctx->o.dim == 3)
    k_pairs<3><<<nb, NTHREADS, 0, st>>>(mode, ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->d_count, nullptr, cnt, nullptr, nullptr, dsub, nsub);
  else
    k_pairs<1><<<nb, NTHREADS, 0, st>>>(mode, ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->d_count, nullptr, cnt, nullptr, nullptr, dsub, nsub);
  unsigned long long total = 0;
  if (np) {
    k_scan_blocks<<<nbk, 1024, 0, st>>>(cnt, np, offs, sums);
    k_scan_sums<<<1, 1024, 0, st>>>(sums, nbk, tot);
    k_scan_add<<<nbk, 1024, 0, st>>>(offs, np, sums);
    CK(cudaMemcpyAsync(&total, tot, 8, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  *n = (size_t)total;
  if (total <= cap && key_i && key_j && total) {
    uint64_t *dki = nullptr, *dkj = nullptr;
    CK(cudaMalloc(&dki, 8 * total));
    CK(cudaMalloc(&dkj, 8 * total));
    if (ctx->o.dim == 3)
      k_pairs<3><<<nb, NTHREADS, 0, st>>>(mode, ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->d_count, offs, cnt, dki, dkj, dsub, nsub);
    else
      k_pairs<1><<<nb, NTHREADS, 0, st>>>(mode, ctx->o, ctx->d_geo, ctx->A, ctx->W, ctx->cs, ctx->d_count, offs, cnt, dki, dkj, dsub, nsub);
    CK(cudaMemcpyAsync(key_i, dki, 8 * total, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(key_j, dkj, 8 * total, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    cudaFree(dki);
    cudaFree(dkj);
  }
  cudaFree(cnt);
  cudaFree(offs);
  cudaFree(sums);
  cudaFree(tot);
  CK(cudaGetLastError());
  return PLUME_OK;
}

int plume_neighbor_pairs(plume_ctx* ctx, int mode, uint64_t* key_i, uint64_t* key_j, size_t cap, size_t* n) {
  return neighbor_pairs(ctx, mode, nullptr, 0, key_i, key_j, cap, n);
}

int plume_neighbor_pairs_of(plume_ctx* ctx, int mode, const uint64_t* keys, size_t nkeys, uint64_t* key_i,
                            uint64_t* key_j, size_t cap, size_t* n) {
  if (!keys && nkeys) return PLUME_E_INVALID;
  static const uint64_t none = 0;
  return neighbor_pairs(ctx, mode, keys ? keys : &none, nkeys, key_i, key_j, cap, n);
}

// ---------------------------------------------------------------- ensembles
int plume_batch_upload(plume_ctx* ctx, const PlumeSoA* host, const uint16_t* member, size_t n) {
  if (!ctx || !member) return PLUME_E_INVALID;
  if (n > ctx->cap) {
    ctx->err = "particle count exceeds capacity";
    return PLUME_E_CAPACITY;
  }
  int rc = copy_soa(ctx, host, 0, n, cudaMemcpyHostToDevice, member);
  if (rc) return rc;
  rc = set_count(ctx, n);
  if (rc) return rc;
  ctx->pending_dead = true;
  return PLUME_OK;
}

int plume_batch_append(plume_ctx* ctx, const PlumeSoA* host, const uint16_t* member, size_t n) {
  if (!ctx || !member) return PLUME_E_INVALID;
  if (ctx->n_alloc + n > ctx->cap) {
    ctx->err = "append exceeds capacity";
    return PLUME_E_CAPACITY;
  }
  int rc = copy_soa(ctx, host, ctx->n_alloc, n, cudaMemcpyHostToDevice, member);
  if (rc) return rc;
  rc = set_count(ctx, ctx->n_alloc + n);
  ctx->pending_dead = true;
  return rc;
}

int plume_batch_download(plume_ctx* ctx, PlumeSoA* host, uint16_t* member, size_t cap, size_t* n) {
  int rc = plume_download(ctx, host, cap, n);
  if (rc) return rc;
  if (member && *n) {
    CK(cudaMemcpy(member, ctx->A.mem, 2 * (*n), cudaMemcpyDeviceToHost));
  }
  return PLUME_OK;
}

// TimeProps::ifend (properties.h:76-79) of member m, or its error status,
// from the host mirror
static bool member_ended(const plume_ctx* ctx, int m) {
  const TimeState& t = ctx->h_ts[m];
  const Opt& o = ctx->hopt[m];
  return (t.time >= o.max_time) || (t.step > o.max_steps) || (ctx->batch && t.status != 0);
}

int plume_batch_time(plume_ctx* ctx, double* time, int* step, int* running, int* status) {
  if (!ctx) return PLUME_E_INVALID;
  CK(cudaStreamSynchronize(ctx->st));
  CK(cudaMemcpy(ctx->h_ts, ctx->ts, sizeof(TimeState) * ctx->nmem, cudaMemcpyDeviceToHost));
  for (int m = 0; m < ctx->nmem; m++) {
    if (time) time[m] = ctx->h_ts[m].time;
    if (step) step[m] = ctx->h_ts[m].step;
    if (running) running[m] = member_ended(ctx, m) ? 0 : 1;
    if (status) status[m] = ctx->h_ts[m].status;
  }
  return PLUME_OK;
}

// captures k steps of the context's stream into one CUDA graph
static int capture_steps(plume_ctx* ctx, int k) {
  if (ctx->gexec) {
    cudaGraphExecDestroy(ctx->gexec);
    ctx->gexec = nullptr;
  }
  const int saved_step = ctx->host_step;
  const unsigned long long saved_launches = ctx->launches;
  ctx->capturing = true;
  CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
  int rc = PLUME_OK;
  for (int q = 0; q < k && rc == PLUME_OK; q++) rc = step_async(ctx);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(ctx->st, &graph);
  ctx->capturing = false;
  ctx->host_step = saved_step;
  ctx->glaunches = ctx->launches - saved_launches;
  ctx->launches = saved_launches;
  if (rc != PLUME_OK || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    if (rc == PLUME_OK) ctx->err = std::string("stream capture: ") + cudaGetErrorString(e);
    return rc != PLUME_OK ? rc : PLUME_E_CUDA;
  }
  e = cudaGraphInstantiate(&ctx->gexec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    ctx->gexec = nullptr;
    ctx->err = std::string("graph instantiate: ") + cudaGetErrorString(e);
    return PLUME_E_CUDA;
  }
  ctx->gsteps = k;
  ctx->gn = ctx->n_alloc;
  return PLUME_OK;
}

int plume_batch_run(plume_ctx* ctx, int max_steps, int graph_steps, int* steps_done) {
  if (!ctx || max_steps < 0 || graph_steps < 0) return PLUME_E_INVALID;
  for (auto& v : ctx->phase_ms) v = 0;
  ctx->launches = 0;
  if (steps_done) *steps_done = 0;
  for (auto& e : ctx->run_ev)
    if (!e) CK(cudaEventCreate(&e));
  int rc = ensure_events(ctx, 1);
  if (rc) return rc;
  ctx->ev = ctx->evs.data();
  int s = ctx_sync_status(ctx);
  if (s) return s;
  // every member stops at its TimeProps::ifend inside the run
  bool refreeze = false;
  for (int m = 0; m < ctx->nmem; m++)
    if (!ctx->h_ts[m].freeze) {
      ctx->h_ts[m].freeze = 1;
      refreeze = true;
    }
  if (refreeze) CK(cudaMemcpy(ctx->ts, ctx->h_ts, sizeof(TimeState) * ctx->nmem, cudaMemcpyHostToDevice));
  bool any = false;
  for (int m = 0; m < ctx->nmem; m++) any |= !member_ended(ctx, m);
  int done = 0;
  CK(cudaEventRecord(ctx->run_ev[0], ctx->st));
  while (any && done < max_steps) {
    const int k = graph_steps > 0 ? std::min(graph_steps, max_steps - done) : 1;
    if (graph_steps > 0) {
      if (!ctx->gexec || ctx->gsteps != k || ctx->n_alloc > ctx->gn) {
        rc = capture_steps(ctx, k);
        if (rc) return rc;
      }
      CK(cudaGraphLaunch(ctx->gexec, ctx->st));
      ctx->host_step += k;
      ctx->launches += ctx->glaunches;
    } else {
      rc = step_async(ctx);
      if (rc) return rc;
    }
    done += k;
    s = finish_steps(ctx);
    if (s) break;
    any = false;
    for (int m = 0; m < ctx->nmem; m++) any |= !member_ended(ctx, m);
  }
  CK(cudaEventRecord(ctx->run_ev[1], ctx->st));
  CK(cudaEventSynchronize(ctx->run_ev[1]));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->run_ev[0], ctx->run_ev[1]);
  ctx->phase_ms[10] = ms;
  if (steps_done) *steps_done = done;
  return s;
}

// ---------------------------------------------------------------- adjoint
static int adj_alloc(plume_ctx* ctx, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    ctx->err = std::string("adjoint storage: ") + cudaGetErrorString(e);
    return PLUME_E_CUDA;
  }
  ctx->adj_allocs.push_back(*p);
  return PLUME_OK;
}
#define AALLOC(ptr, bytes)                                            \
  do {                                                                \
    int rc_ = adj_alloc(ctx, (void**)&(ptr), (bytes));                \
    if (rc_) return rc_;                                              \
  } while (0)

static int alloc_dev_adj(plume_ctx* ctx, Dev& D, size_t n) {
  AALLOC(D.key, 8 * n);
  double** f[] = {&D.x, &D.y, &D.z, &D.vx, &D.vy, &D.vz, &D.vsx, &D.vsy, &D.vsz, &D.mass,
                  &D.h, &D.rho, &D.e, &D.p, &D.Y, &D.gam, &D.c, &D.T, &D.cp};
  for (auto p : f) AALLOC(*p, 8 * n);
  AALLOC(D.phase, n);
  AALLOC(D.bc, n);
  AALLOC(D.inv, n);
  AALLOC(D.bkt, 4 * n);
  AALLOC(D.mem, 2 * n);
  return PLUME_OK;
}
static int alloc_adj(plume_ctx* ctx, Adj& B, size_t n) {
  double** f[] = {&B.x, &B.y, &B.z, &B.vx, &B.vy, &B.vz, &B.vsx, &B.vsy, &B.vsz,
                  &B.m, &B.h, &B.rho, &B.e, &B.p, &B.Y, &B.c, &B.T, &B.cp};
  for (auto p : f) AALLOC(*p, 8 * n);
  return PLUME_OK;
}
static void zero_adj(const Adj& B, size_t n, cudaStream_t st) {
  double* const f[18] = {B.x, B.y, B.z, B.vx, B.vy, B.vz, B.vsx, B.vsy, B.vsz,
                         B.m, B.h, B.rho, B.e, B.p, B.Y, B.c, B.T, B.cp};
  for (auto p : f) cudaMemsetAsync(p, 0, 8 * n, st);
}
static int alloc_rec(plume_ctx* ctx, AdjRec& r, size_t n) {
  r = AdjRec{};
  int rc = alloc_dev_adj(ctx, r.S, n);
  if (rc) return rc;
  const int nl = ctx->opt.num_loop > 0 ? ctx->opt.num_loop : 1;
  AALLOC(r.h1, 8 * n);
  AALLOC(r.hit, 8 * n * (size_t)(nl + 1));
  AALLOC(r.nit, n);
  double** d[] = {&r.v1x, &r.v1y, &r.v1z, &r.e1, &r.rho2, &r.Y2, &r.e2, &r.vs3x, &r.vs3y, &r.vs3z,
                  &r.wnd, &r.wnv};
  for (auto p : d) AALLOC(*p, 8 * n);
  AALLOC(r.bc3, n);
  AALLOC(r.perm, 4 * n);
  AALLOC(r.L.e, sizeof(uint2) * (size_t)LCAP * n);
  AALLOC(r.L.cnt, sizeof(uint16_t) * n);
  AALLOC(r.real_idx, 4 * n);
  AALLOC(r.d_real, sizeof(int));
  AALLOC(r.cs, 4 * ((size_t)ctx->ncells + 2));
  AALLOC(r.h27, 8 * (size_t)ctx->nbk);
  AALLOC(r.ts, sizeof(TimeState));
  AALLOC(r.argmin, sizeof(int));
  AALLOC(r.d_count, sizeof(int));
  return PLUME_OK;
}
static void save_ckpt(plume_ctx* ctx, AdjCkpt& c) {
  copy_dev(c.A, ctx->A, ctx->n_alloc, ctx->st);
  dcopy(c.d_count, ctx->d_count, sizeof(int), ctx->st);
  dcopy(c.ts, ctx->ts, sizeof(TimeState), ctx->st);
  c.n_alloc = ctx->n_alloc;
  c.host_step = ctx->host_step;
}
static int restore_ckpt(plume_ctx* ctx, const AdjCkpt& c) {
  copy_dev(ctx->A, c.A, c.n_alloc, ctx->st);
  dcopy(ctx->d_count, c.d_count, sizeof(int), ctx->st);
  dcopy(ctx->ts, c.ts, sizeof(TimeState), ctx->st);
  ctx->n_alloc = c.n_alloc;
  ctx->host_step = c.host_step;
  CK(cudaMemcpyAsync(ctx->d_hstep, &ctx->host_step, sizeof(int), cudaMemcpyHostToDevice, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  ctx->pending_dead = true;
  return PLUME_OK;
}

// scratch of the backward of one step
struct AdjTmp {
  double *ox, *oy, *oz, *oe, *orho, *oY, *oh;
  double *dtbar, *ng0bar;
};

// backward of one recorded step: adjoints `cur` (sorted order of the step,
// i.e. the order of the state after it) -> `prev` (order before its sort)
static int adj_step_back(plume_ctx* ctx, const AdjRec& r, const TimeState& hts, int nlive, Adj& cur, Adj& prev,
                         const AdjTmp& t) {
  cudaStream_t st = ctx->st;
  const int n = (int)ctx->adj_rows;
  const int nb = nblocks(n ? n : 1);
  const Opt& o = ctx->o;
  const Geo& g = ctx->hgeo[0];
  const double dt = hts.dtime;
  const bool lans = o.lans != 0;
  CK(cudaMemsetAsync(t.dtbar, 0, sizeof(double), st));
  Work Wv{};
  Wv.hlist = r.S.h;  // h at the search
  Packed K{};
  // P
  k_adj_pos<<<nb, NTHREADS, 0, st>>>(r.S, r.bc3, r.vs3x, r.vs3y, r.vs3z, r.v1x, r.v1y, r.v1z, n, dt,
                                     hts.erupt, lans ? 1 : 0, cur, t.dtbar);
  AdjIn in{};
  in.dtbar = t.dtbar;
  in.ng0bar = t.ng0bar;
  // V: reads v after M, rho after D, h after A
  if (lans) {
    k_adj_vel_pre<<<nb, NTHREADS, 0, st>>>(r.S, n, cur, t.ox, t.oy, t.oz);
    Dev Sv = r.S;
    Sv.h = r.h1;
    Sv.rho = r.rho2;
    Sv.vx = r.v1x; Sv.vy = r.v1y; Sv.vz = r.v1z;
    AdjIn iv = in;
    iv.vsx = t.ox; iv.vsy = t.oy; iv.vsz = t.oz;
    iv.vsx_new = r.vs3x; iv.vsy_new = r.vs3y; iv.vsz_new = r.vs3z;
    iv.wnv = r.wnv;
    k_adj_sweep<VVel><<<nb, NTHREADS, 0, st>>>(o, g, Sv, Wv, K, r.cs, r.h27, r.d_real, r.real_idx, ctx->ts,
                                               r.L, cur, iv, dt);
  }
  // D: reads rho before D, e after M, h after A
  {
    k_adj_dens_pre<<<nb, NTHREADS, 0, st>>>(o, r.S, r.rho2, r.Y2, r.e2, n, cur, t.orho, t.oY, t.oe, t.ng0bar);
    Dev Sd = r.S;
    Sd.h = r.h1;
    Sd.e = r.e1;
    AdjIn id = in;
    id.rho = t.orho; id.Y = t.oY; id.ee = t.oe;
    id.rho_new = r.rho2; id.Y_new = r.Y2; id.e_new = r.e2;
    id.wnd = r.wnd;
    k_adj_sweep<VDens><<<nb, NTHREADS, 0, st>>>(o, g, Sd, Wv, K, r.cs, r.h27, r.d_real, r.real_idx, ctx->ts,
                                                r.L, cur, id, dt);
  }
  // M: reads the state after the sort with h after A
  {
    k_adj_mom_pre<<<nb, NTHREADS, 0, st>>>(r.S, n, cur, t.ox, t.oy, t.oz, t.oe);
    Dev Sm = r.S;
    Sm.h = r.h1;
    AdjIn im = in;
    im.vx = t.ox; im.vy = t.oy; im.vz = t.oz; im.e = t.oe;
    k_adj_sweep<VMom><<<nb, NTHREADS, 0, st>>>(o, g, Sm, Wv, K, r.cs, r.h27, r.d_real, r.real_idx, ctx->ts,
                                               r.L, cur, im, dt);
  }
  // A
  if (r.adaptive) {
    k_adj_adapt_pre<<<nb, NTHREADS, 0, st>>>(r.S, r.nit, n, cur, t.oh);
    k_adj_adaptive<<<nb, NTHREADS, 0, st>>>(o, g, r.S, Wv, r.cs, n, r.hit, r.nit, n, t.oh, cur);
  }
  // dt (state before the step: h before A, c)
  k_adj_dt<<<1, 1, 0, st>>>(r.S, r.argmin, o.cfl, t.dtbar, cur);
  // back to the order before the sort
  zero_adj(prev, (size_t)n, st);
  if (nlive > 0) k_adj_unperm<<<nblocks(nlive), NTHREADS, 0, st>>>(cur, prev, r.perm, nlive);
  std::swap(cur, prev);
  CK(cudaGetLastError());
  return PLUME_OK;
}

int plume_adjoint_record(plume_ctx* ctx, int nsteps, int checkpoint_every) {
  if (!ctx || nsteps < 1 || checkpoint_every < 1) return PLUME_E_INVALID;
  if (ctx->nmem != 1 || ctx->o.dim != 3 || ctx->opt.precision != PLUME_PREC_FP64 ||
      ctx->opt.kernel != PLUME_KERNEL_GAUSS || !ctx->use_lists) {
    ctx->err = "adjoint: one 3D FP64 run with the Gaussian kernel and neighbour lists";
    return PLUME_E_INVALID;
  }
  if (ctx->nimg) {
    ctx->err = "adjoint: the wall boundary is not differentiated (clear the wall images)";
    return PLUME_E_INVALID;
  }
  if (ctx->o.method != PLUME_METHOD_SPH) {
    ctx->err = "adjoint: the GSPH step is not differentiated";
    return PLUME_E_INVALID;
  }
  if (ctx->inlet_reserve) {
    ctx->err = "adjoint: the inlet is not differentiated (clear it)";
    return PLUME_E_INVALID;
  }
  for (void* p : ctx->adj_allocs) cudaFree(p);
  ctx->adj_allocs.clear();
  ctx->ckpts.clear();
  ctx->recs.clear();
  if (ctx->pending_dead) {  // the recorded window starts from a sorted state
    int rc = search(ctx);
    if (rc) return rc;
    int s = finish_steps(ctx);
    if (s) return s;
  }
  const size_t n = ctx->n_alloc;
  ctx->adj_rows = n;
  ctx->adj_every = checkpoint_every;
  ctx->adj_steps = nsteps;
  const int nseg = (nsteps + checkpoint_every - 1) / checkpoint_every;
  ctx->ckpts.resize((size_t)nseg + 1);
  for (auto& c : ctx->ckpts) {
    int rc = alloc_dev_adj(ctx, c.A, n);
    if (rc) return rc;
    AALLOC(c.d_count, sizeof(int));
    AALLOC(c.ts, sizeof(TimeState));
  }
  for (auto& v : ctx->phase_ms) v = 0;
  ctx->launches = 0;
  int rc = ensure_events(ctx, 1);
  if (rc) return rc;
  ctx->ev = ctx->evs.data();
  for (int k = 0; k < nsteps; k++) {
    if (k % checkpoint_every == 0) save_ckpt(ctx, ctx->ckpts[(size_t)(k / checkpoint_every)]);
    rc = step_async(ctx);
    if (rc) return rc;
  }
  // the window keeps the row count of its start (deleted rows sort last)
  CK(cudaStreamSynchronize(ctx->st));
  save_ckpt(ctx, ctx->ckpts.back());
  int s = finish_steps(ctx);
  ctx->ckpts.back().n_alloc = n;
  return s;
}

// PlumeSoA field k of the adjoint field order of Adj
static double* soa_field(const PlumeSoA* s, int f) {
  double* const p[18] = {s->x, s->y, s->z, s->vx, s->vy, s->vz, s->vsx, s->vsy, s->vsz,
                         s->mass, s->h, s->rho, s->e, s->p, s->Y, s->c, s->T, s->cp};
  return p[f];
}
static double* adj_field(const Adj& B, int f) {
  double* const p[18] = {B.x, B.y, B.z, B.vx, B.vy, B.vz, B.vsx, B.vsy, B.vsz,
                         B.m, B.h, B.rho, B.e, B.p, B.Y, B.c, B.T, B.cp};
  return p[f];
}

int plume_adjoint_backward(plume_ctx* ctx, const PlumeSoA* final_bar, size_t n_final, PlumeSoA* initial_bar,
                           size_t cap, size_t* n_initial, double* ng0_bar) {
  if (!ctx || !final_bar || !final_bar->key || !initial_bar || !initial_bar->key || !n_initial)
    return PLUME_E_INVALID;
  if (ctx->ckpts.empty()) {
    ctx->err = "adjoint: no recorded window (plume_adjoint_record)";
    return PLUME_E_INVALID;
  }
  const size_t n = ctx->adj_rows;
  const AdjCkpt& c0 = ctx->ckpts.front();
  *n_initial = c0.n_alloc;
  if (c0.n_alloc > cap) {
    ctx->err = "adjoint: initial_bar capacity too small";
    return PLUME_E_CAPACITY;
  }
  cudaStream_t st = ctx->st;
  // storage of the backward (kept for further calls)
  const int every = ctx->adj_every;
  if (ctx->recs.empty()) {
    ctx->recs.resize((size_t)every);
    for (auto& r : ctx->recs) {
      int rc = alloc_rec(ctx, r, n);
      if (rc) return rc;
    }
  }
  Adj cur{}, prev{};
  AdjTmp t{};
  {
    int rc;
    if ((rc = alloc_adj(ctx, cur, n)) || (rc = alloc_adj(ctx, prev, n))) return rc;
    double** tp[] = {&t.ox, &t.oy, &t.oz, &t.oe, &t.orho, &t.oY, &t.oh};
    for (auto p : tp) AALLOC(*p, 8 * n);
    AALLOC(t.dtbar, sizeof(double));
    AALLOC(t.ng0bar, sizeof(double));
  }
  // adjoint of the final state, by key, in the final state's rows
  {
    const AdjCkpt& cf = ctx->ckpts.back();
    std::vector<uint64_t> keys(n);
    std::vector<uint8_t> bc(n);
    CK(cudaMemcpy(keys.data(), cf.A.key, 8 * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(bc.data(), cf.A.bc, n, cudaMemcpyDeviceToHost));
    std::vector<std::pair<uint64_t, uint32_t>> kr;
    kr.reserve(n);
    for (size_t r = 0; r < n; r++)
      if (bc[r] != BC_DEAD) kr.push_back({keys[r], (uint32_t)r});
    std::sort(kr.begin(), kr.end());
    std::vector<double> h(18 * n, 0.0);
    for (size_t q = 0; q < n_final; q++) {
      auto it = std::lower_bound(kr.begin(), kr.end(), std::make_pair(final_bar->key[q], (uint32_t)0));
      if (it == kr.end() || it->first != final_bar->key[q]) continue;  // not in the final state
      for (int f = 0; f < 18; f++) {
        const double* src = soa_field(final_bar, f);
        if (src) h[(size_t)f * n + it->second] = src[q];
      }
    }
    for (int f = 0; f < 18; f++)
      CK(cudaMemcpy(adj_field(cur, f), h.data() + (size_t)f * n, 8 * n, cudaMemcpyHostToDevice));
  }
  CK(cudaMemset(t.ng0bar, 0, sizeof(double)));
  const int nseg = (int)ctx->ckpts.size() - 1;
  std::vector<TimeState> hts((size_t)every);
  std::vector<int> nlive((size_t)every);
  for (int seg = nseg - 1; seg >= 0; seg--) {
    int rc = restore_ckpt(ctx, ctx->ckpts[(size_t)seg]);
    if (rc) return rc;
    const int len = std::min(every, ctx->adj_steps - seg * every);
    for (int k = 0; k < len; k++) {
      ctx->rec = &ctx->recs[(size_t)k];
      rc = step_async(ctx);
      ctx->rec = nullptr;
      if (rc) return rc;
    }
    CK(cudaStreamSynchronize(st));
    for (int k = 0; k < len; k++) {
      CK(cudaMemcpy(&hts[(size_t)k], ctx->recs[(size_t)k].ts, sizeof(TimeState), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(&nlive[(size_t)k], ctx->recs[(size_t)k].d_count, sizeof(int), cudaMemcpyDeviceToHost));
      double dtmin;
      memcpy(&dtmin, &hts[(size_t)k].dtmin_bits, sizeof(double));
      if (hts[(size_t)k].status) {
        ctx->err = "adjoint: recomputed step failed with status " + std::to_string(hts[(size_t)k].status);
        return hts[(size_t)k].status;
      }
      if (hts[(size_t)k].dtime != ctx->o.cfl * dtmin) {
        ctx->err = "adjoint: dt clipped to an output or end time inside the window";
        return PLUME_E_INVALID;
      }
    }
    for (int k = len - 1; k >= 0; k--) {
      rc = adj_step_back(ctx, ctx->recs[(size_t)k], hts[(size_t)k], nlive[(size_t)k], cur, prev, t);
      if (rc) return rc;
    }
  }
  CK(cudaStreamSynchronize(st));
  // rows of the window's first state
  {
    const size_t n0 = c0.n_alloc;
    CK(cudaMemcpy(initial_bar->key, c0.A.key, 8 * n0, cudaMemcpyDeviceToHost));
    for (int f = 0; f < 18; f++) {
      double* dst = soa_field(initial_bar, f);
      if (dst) CK(cudaMemcpy(dst, adj_field(cur, f), 8 * n0, cudaMemcpyDeviceToHost));
    }
  }
  if (ng0_bar) CK(cudaMemcpy(ng0_bar, t.ng0bar, sizeof(double), cudaMemcpyDeviceToHost));
  // the context continues from the window's final state
  int rc = restore_ckpt(ctx, ctx->ckpts.back());
  if (rc) return rc;
  return finish_steps(ctx);
}

// ---------------------------------------------------------------- snapshots
int plume_snapshot_begin(plume_ctx* ctx, PlumeSoA* host, size_t cap) {
  if (!ctx || !host) return PLUME_E_INVALID;
  const bool d3 = ctx->o.dim == 3;
  if (!host->key || !host->x || !host->vx || !host->rho || !host->e || !host->Y || !host->p || !host->mass ||
      !host->h || !host->phase || !host->bc_type || (d3 && (!host->y || !host->z || !host->vy || !host->vz))) {
    ctx->err = "snapshot: missing host array";
    return PLUME_E_INVALID;
  }
  if (ctx->nmem != 1) {
    ctx->err = "snapshot: single-run contexts only";
    return PLUME_E_INVALID;
  }
  if (ctx->snap_busy) {
    ctx->err = "snapshot: one in flight (plume_snapshot_end first)";
    return PLUME_E_INVALID;
  }
  size_t nt = 0;
  int rc = plume_count(ctx, &nt, nullptr);  // drops deleted rows
  if (rc) return rc;
  if (nt > cap) {
    ctx->err = "snapshot capacity too small";
    return PLUME_E_CAPACITY;
  }
  if (!ctx->snap_st) {
    CK(cudaStreamCreateWithFlags(&ctx->snap_st, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ctx->snap_staged, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ctx->snap_done, cudaEventDisableTiming));
    CK(cudaMallocHost(&ctx->snap_ts, sizeof(TimeState)));
  }
  if (ctx->snap_cap < nt) {
    void* sp[] = {ctx->snap.key, ctx->snap.x, ctx->snap.y, ctx->snap.z, ctx->snap.vx, ctx->snap.vy, ctx->snap.vz,
                  ctx->snap.mass, ctx->snap.h, ctx->snap.rho, ctx->snap.e, ctx->snap.p, ctx->snap.Y,
                  ctx->snap.phase, ctx->snap.bc, ctx->snap.inv};
    for (void* q : sp) if (q) cudaFree(q);
    ctx->snap = Dev{};
    const size_t c = std::max(nt, (size_t)1);
    double** dd[] = {&ctx->snap.x, &ctx->snap.y, &ctx->snap.z, &ctx->snap.vx, &ctx->snap.vy, &ctx->snap.vz,
                     &ctx->snap.mass, &ctx->snap.h, &ctx->snap.rho, &ctx->snap.e, &ctx->snap.p, &ctx->snap.Y};
    CK(cudaMalloc(&ctx->snap.key, 8 * c));
    for (double** q : dd) CK(cudaMalloc(q, 8 * c));
    CK(cudaMalloc(&ctx->snap.phase, c));
    CK(cudaMalloc(&ctx->snap.bc, c));
    CK(cudaMalloc(&ctx->snap.inv, c));
    ctx->snap_cap = c;
  }
  // stage on the main stream (later steps overwrite the table in place)
  cudaStream_t st = ctx->st;
  Dev& A = ctx->A;
  Dev& S = ctx->snap;
  std::vector<CopyJob> stage = {
      {(char*)S.key, (const char*)A.key, 8 * nt},   {(char*)S.x, (const char*)A.x, 8 * nt},
      {(char*)S.vx, (const char*)A.vx, 8 * nt},     {(char*)S.mass, (const char*)A.mass, 8 * nt},
      {(char*)S.h, (const char*)A.h, 8 * nt},       {(char*)S.rho, (const char*)A.rho, 8 * nt},
      {(char*)S.e, (const char*)A.e, 8 * nt},       {(char*)S.p, (const char*)A.p, 8 * nt},
      {(char*)S.Y, (const char*)A.Y, 8 * nt},       {(char*)S.phase, (const char*)A.phase, nt},
      {(char*)S.bc, (const char*)A.bc, nt},         {(char*)S.inv, (const char*)A.inv, nt}};
  if (d3) {
    stage.push_back({(char*)S.y, (const char*)A.y, 8 * nt});
    stage.push_back({(char*)S.z, (const char*)A.z, 8 * nt});
    stage.push_back({(char*)S.vy, (const char*)A.vy, 8 * nt});
    stage.push_back({(char*)S.vz, (const char*)A.vz, 8 * nt});
  }
  if (nt) {
    CopyJobs J{};
    for (const CopyJob& c : stage) J.j[J.n++] = c;
    k_copy_multi<<<dim3(2 * 152, J.n), 256, 0, st>>>(J);
    CK(cudaGetLastError());
  }
  CK(cudaMemcpyAsync(ctx->snap_ts, ctx->ts, sizeof(TimeState), cudaMemcpyDeviceToHost, st));
  CK(cudaEventRecord(ctx->snap_staged, st));
  // then to the host on the side stream
  CK(cudaStreamWaitEvent(ctx->snap_st, ctx->snap_staged, 0));
  std::vector<CopyJob> out = {
      {(char*)host->key, (const char*)S.key, 8 * nt},   {(char*)host->x, (const char*)S.x, 8 * nt},
      {(char*)host->vx, (const char*)S.vx, 8 * nt},     {(char*)host->mass, (const char*)S.mass, 8 * nt},
      {(char*)host->h, (const char*)S.h, 8 * nt},       {(char*)host->rho, (const char*)S.rho, 8 * nt},
      {(char*)host->e, (const char*)S.e, 8 * nt},       {(char*)host->p, (const char*)S.p, 8 * nt},
      {(char*)host->Y, (const char*)S.Y, 8 * nt},       {(char*)host->phase, (const char*)S.phase, nt},
      {(char*)host->bc_type, (const char*)S.bc, nt}};
  if (host->involved) out.push_back({(char*)host->involved, (const char*)S.inv, nt});
  if (d3) {
    out.push_back({(char*)host->y, (const char*)S.y, 8 * nt});
    out.push_back({(char*)host->z, (const char*)S.z, 8 * nt});
    out.push_back({(char*)host->vy, (const char*)S.vy, 8 * nt});
    out.push_back({(char*)host->vz, (const char*)S.vz, 8 * nt});
  }
  if (nt) {
    // page-locked host arrays: one kernel writes them; else DMA per field
    CopyJobs J{};
    bool mapped = true;
    for (CopyJob c : out) {
      void* dp = mapped_host(c.dst);
      if (!dp) { mapped = false; break; }
      c.dst = (char*)dp;
      J.j[J.n++] = c;
    }
    if (mapped) {
      k_copy_multi<<<dim3(2 * 152, J.n), 256, 0, ctx->snap_st>>>(J);
      CK(cudaGetLastError());
    } else {
      for (const CopyJob& c : out) CK(cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyDeviceToHost, ctx->snap_st));
    }
  }
  CK(cudaEventRecord(ctx->snap_done, ctx->snap_st));
  ctx->snap_n = nt;
  ctx->snap_busy = true;
  return PLUME_OK;
}

int plume_snapshot_end(plume_ctx* ctx, size_t* n, double* time, int* step) {
  if (!ctx) return PLUME_E_INVALID;
  if (!ctx->snap_busy) {
    ctx->err = "snapshot: none in flight";
    return PLUME_E_INVALID;
  }
  CK(cudaEventSynchronize(ctx->snap_done));
  CK(cudaEventSynchronize(ctx->snap_staged));
  ctx->snap_busy = false;
  if (n) *n = ctx->snap_n;
  if (time) *time = ctx->snap_ts->time;
  if (step) *step = ctx->snap_ts->step;
  return PLUME_OK;
}

// ---------------------------------------------------------------- domain growth
int plume_set_bucket_involvement(plume_ctx* ctx, const uint8_t* state, size_t nbuckets) {
  if (!ctx || !state) return PLUME_E_INVALID;
  if (!ctx->binv || nbuckets != (size_t)ctx->nbk) {
    ctx->err = "bucket involvement: 3D only, one state per bucket of the context";
    return PLUME_E_INVALID;
  }
  for (size_t b = 0; b < nbuckets; b++)
    if (state[b] > PLUME_BINV_BOTH) {
      ctx->err = "bucket involvement: states are 0..3";
      return PLUME_E_INVALID;
    }
  CK(cudaMemcpyAsync(ctx->binv, state, nbuckets, cudaMemcpyHostToDevice, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return PLUME_OK;
}

int plume_get_bucket_involvement(plume_ctx* ctx, uint8_t* state, size_t nbuckets) {
  if (!ctx || !state) return PLUME_E_INVALID;
  if (!ctx->binv || nbuckets != (size_t)ctx->nbk) {
    ctx->err = "bucket involvement: 3D only, one state per bucket of the context";
    return PLUME_E_INVALID;
  }
  CK(cudaMemcpyAsync(state, ctx->binv, nbuckets, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return PLUME_OK;
}

int plume_scan_outside_layer(plume_ctx* ctx, int* adapt) {
  if (!ctx || !adapt) return PLUME_E_INVALID;
  if (!ctx->binv) {
    ctx->err = "scan_outside_layer: 3D only";
    return PLUME_E_INVALID;
  }
  int rc = search(ctx);  // bucket contents of the current positions
  if (rc) return rc;
  cudaStream_t st = ctx->st;
  cudaMemsetAsync(ctx->d_adapt, 0, sizeof(int) * (size_t)ctx->nmem, st);
  k_scan_outside<<<nblocks(ctx->nbk), NTHREADS, 0, st>>>(ctx->d_geo, ctx->bmember, ctx->A, ctx->cs, ctx->binv,
                                                         ctx->bflags, ctx->bface, ctx->nbk, ctx->explicit_types,
                                                         ctx->d_adapt);
  std::vector<int> a((size_t)ctx->nmem);
  CK(cudaMemcpyAsync(a.data(), ctx->d_adapt, sizeof(int) * (size_t)ctx->nmem, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  int sum = 0;
  for (int v : a) sum += v;
  *adapt = sum;
  return PLUME_OK;
}

int plume_adapt_domain(plume_ctx* ctx) {
  if (!ctx) return PLUME_E_INVALID;
  if (!ctx->binv) {
    ctx->err = "adapt_domain: 3D only";
    return PLUME_E_INVALID;
  }
  int rc = search(ctx);
  if (rc) return rc;
  cudaStream_t st = ctx->st;
  k_adapt_buckets<<<nblocks(ctx->nbk), NTHREADS, 0, st>>>(ctx->d_geo, ctx->bmember, ctx->cs, ctx->binv, ctx->bflags,
                                                          ctx->bface, ctx->nbk, ctx->explicit_types, ctx->bmark);
  const int n = (int)ctx->n_alloc;
  k_adapt_particles<<<nblocks(n ? n : 1), NTHREADS, 0, st>>>(ctx->d_geo, ctx->A, ctx->d_count, ctx->bmark,
                                                             ctx->bflags, ctx->bface, ctx->explicit_types);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  return PLUME_OK;
}

// kind 0: add_pressure_ghost, kind 1: add_wall_ghost, kind 2: add_air
static int add_ghost_layers(plume_ctx* ctx, const PlumeAtmosphere* atm, uint64_t key_base, size_t* added, int kind) {
  const char* name = kind == 0 ? "add_pressure_ghost" : (kind == 1 ? "add_wall_ghost" : "add_air");
  if (!ctx || !atm || !added) return PLUME_E_INVALID;
  *added = 0;
  if (!ctx->binv) {
    ctx->err = std::string(name) + ": 3D only";
    return PLUME_E_INVALID;
  }
  if (ctx->nmem != 1) {
    ctx->err = std::string(name) + ": single-run contexts only";
    return PLUME_E_INVALID;
  }
  const double dx = ctx->opt.sml_phase2;
  const double ground = ctx->hgeo[0].lo[2];
  if (!(dx > 0) || ctx->hgeo[0].del / dx > 1024.0) {
    ctx->err = std::string(name) + ": bucket edge / smoothing length must be in (0, 1024]";
    return PLUME_E_INVALID;
  }
  int rc = search(ctx);
  if (rc) return rc;
  cudaStream_t st = ctx->st;
  const int nbk = ctx->nbk;
  uint32_t* cnt = nullptr;
  unsigned long long* offs = nullptr;
  ScratchFree scratch;
  CK(cudaMalloc(&cnt, 4 * (size_t)nbk));
  scratch.p[0] = cnt;
  CK(cudaMalloc(&offs, 8 * (size_t)nbk));
  scratch.p[1] = offs;
  k_pg_buckets<<<nblocks(nbk), NTHREADS, 0, st>>>(ctx->d_geo, ctx->A, ctx->cs, ctx->binv, ctx->bflags, ctx->bface,
                                                 nbk, ctx->explicit_types, kind, dx, ground, cnt);
  CK(cudaGetLastError());
  std::vector<uint32_t> hc((size_t)nbk);
  std::vector<unsigned long long> ho((size_t)nbk);
  CK(cudaMemcpyAsync(hc.data(), cnt, 4 * (size_t)nbk, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  unsigned long long tot = 0;
  for (int b = 0; b < nbk; b++) {
    ho[b] = tot;
    tot += hc[b];
  }
  if (ctx->n_alloc + tot > ctx->cap) {
    ctx->err = std::string(name) + " exceeds capacity";
    return PLUME_E_CAPACITY;
  }
  if (tot) {
    CK(cudaMemcpyAsync(offs, ho.data(), 8 * (size_t)nbk, cudaMemcpyHostToDevice, st));
    const Atm a{atm->Ta0,  atm->pa0,  atm->Ra,   atm->gamma, atm->H1,   atm->H2,   atm->H3,   atm->miu1, atm->miu2,
                atm->Ata1, atm->Ate1, atm->Ata2, atm->Atb2,  atm->Ata3, atm->Atb3, atm->AtC3, atm->Ate3};
    k_pg_fill<<<nbk, 128, 0, st>>>(ctx->d_geo, ctx->d_opt, ctx->A, ctx->cs, ctx->binv, ctx->bflags, ctx->bface,
                                  ctx->explicit_types, kind, cnt, offs, a, dx, ground, ctx->n_alloc,
                                  (unsigned long long)key_base);
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(st));
  ctx->launches += tot ? 2 : 1;
  if (tot) {
    rc = set_count(ctx, ctx->n_alloc + (size_t)tot);
    if (rc) return rc;
    ctx->pending_dead = true;
  }
  *added = (size_t)tot;
  return PLUME_OK;
}

int plume_add_pressure_ghost(plume_ctx* ctx, const PlumeAtmosphere* atm, uint64_t key_base, size_t* added) {
  return add_ghost_layers(ctx, atm, key_base, added, 0);
}

int plume_add_wall_ghost(plume_ctx* ctx, const PlumeAtmosphere* atm, uint64_t key_base, size_t* added) {
  return add_ghost_layers(ctx, atm, key_base, added, 1);
}

int plume_add_air(plume_ctx* ctx, const PlumeAtmosphere* atm, uint64_t key_base, size_t* added) {
  return add_ghost_layers(ctx, atm, key_base, added, 2);
}

// ---------------------------------------------------------------- GSPH
int plume_gsph_gradients(plume_ctx* ctx, uint64_t* key, double* grad, size_t cap, size_t* n) {
  if (!ctx || !n) return PLUME_E_INVALID;
  if (!ctx->grad || !ctx->grad_valid) {
    ctx->err = "GSPH gradients: none computed by the last step";
    return PLUME_E_INVALID;
  }
  int cnt = 0;
  CK(cudaMemcpyAsync(&cnt, ctx->d_count, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  *n = (size_t)cnt;
  if (cap < (size_t)cnt) return PLUME_OK;
  if (!key || !grad) return PLUME_E_INVALID;
  const size_t per = (size_t)((ctx->o.dim + 2) * ctx->o.dim);
  std::vector<uint8_t> bc((size_t)cnt);
  std::vector<uint64_t> k((size_t)cnt);
  std::vector<double> g((size_t)cnt * per);
  if (cnt) {
    CK(cudaMemcpyAsync(bc.data(), ctx->A.bc, (size_t)cnt, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(k.data(), ctx->A.key, 8 * (size_t)cnt, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(g.data(), ctx->grad, 8 * (size_t)cnt * per, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  // rows of the last step; rows deleted by it are left out
  size_t r = 0;
  for (int i = 0; i < cnt; i++) {
    if (bc[i] == BC_DEAD) continue;
    key[r] = k[i];
    memcpy(grad + r * per, g.data() + (size_t)i * per, 8 * per);
    r++;
  }
  *n = r;
  return PLUME_OK;
}

// ---------------------------------------------------------------- wall boundary
int plume_set_wall_images(plume_ctx* ctx, const uint64_t* ghost_keys, const double* image_xyz, size_t n) {
  if (!ctx || (n && (!ghost_keys || !image_xyz))) return PLUME_E_INVALID;
  if (ctx->o.dim != 3) {
    ctx->err = "wall images: 3D only";
    return PLUME_E_INVALID;
  }
  if (n > (size_t)0x7fffffff) return PLUME_E_CAPACITY;
  if (ctx->img_key) { cudaFree(ctx->img_key); ctx->img_key = nullptr; }
  if (ctx->img_xyz) { cudaFree(ctx->img_xyz); ctx->img_xyz = nullptr; }
  if (ctx->bc_map) { cudaFree(ctx->bc_map); ctx->bc_map = nullptr; }
  ctx->nimg = 0;
  if (n == 0) return PLUME_OK;
  std::vector<size_t> ord(n);
  for (size_t i = 0; i < n; i++) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return ghost_keys[a] < ghost_keys[b]; });
  std::vector<uint64_t> k(n);
  std::vector<double> x(3 * n);
  for (size_t r = 0; r < n; r++) {
    k[r] = ghost_keys[ord[r]];
    for (int a = 0; a < 3; a++) x[3 * r + a] = image_xyz[3 * ord[r] + a];
    if (r && k[r] == k[r - 1]) {
      ctx->err = "wall images: a ghost key twice";
      return PLUME_E_INVALID;
    }
  }
  CK(cudaMalloc(&ctx->img_key, 8 * n));
  CK(cudaMalloc(&ctx->img_xyz, 24 * n));
  CK(cudaMemcpy(ctx->img_key, k.data(), 8 * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->img_xyz, x.data(), 24 * n, cudaMemcpyHostToDevice));
  // one slot per (member, image)
  if ((size_t)ctx->nmem * n > (size_t)0x7fffffff) return PLUME_E_CAPACITY;
  CK(cudaMalloc(&ctx->bc_map, sizeof(int) * (size_t)ctx->nmem * n));
  ctx->nimg = (int)n;
  return PLUME_OK;
}

int plume_search_bnd_images(plume_ctx* ctx, size_t* n_out) {
  if (!ctx || !n_out) return PLUME_E_INVALID;
  *n_out = 0;
  if (ctx->o.dim != 3 || ctx->nmem != 1) {
    ctx->err = "search_bnd_images: single-run 3D contexts only";
    return PLUME_E_INVALID;
  }
  int rc = search(ctx);
  if (rc) return rc;
  cudaStream_t st = ctx->st;
  const Geo& g = ctx->hgeo[0];
  const double zmax = g.mind[2] + g.nb[2] * g.del - g.mind[2];  // len_domain in z
  const unsigned int cap = (unsigned int)std::min<size_t>(ctx->n_alloc ? ctx->n_alloc : 1, 0x7fffffff);
  unsigned long long* dk = nullptr;
  double* dx = nullptr;
  unsigned int* dn = nullptr;
  ScratchFree scratch;
  CK(cudaMalloc(&dk, 8 * (size_t)cap));
  scratch.p[0] = dk;
  CK(cudaMalloc(&dx, 24 * (size_t)cap));
  scratch.p[1] = dx;
  CK(cudaMalloc(&dn, sizeof(unsigned int)));
  scratch.p[2] = dn;
  CK(cudaMemsetAsync(dn, 0, sizeof(unsigned int), st));
  const int n = (int)ctx->n_alloc;
  k_find_images<<<nblocks(n ? n : 1), NTHREADS, 0, st>>>(ctx->d_geo, ctx->A, ctx->d_count, ctx->bflags, ctx->bface,
                                                         ctx->explicit_types, zmax, dk, dx, dn, cap);
  ctx->launches++;
  CK(cudaGetLastError());
  unsigned int cnt = 0;
  CK(cudaMemcpyAsync(&cnt, dn, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  cnt = std::min(cnt, cap);
  std::vector<uint64_t> k(cnt);
  std::vector<double> x(3 * (size_t)cnt);
  if (cnt) {
    CK(cudaMemcpyAsync(k.data(), dk, 8 * (size_t)cnt, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(x.data(), dx, 24 * (size_t)cnt, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  rc = plume_set_wall_images(ctx, k.data(), x.data(), cnt);
  if (rc) return rc;
  *n_out = cnt;
  return PLUME_OK;
}

int plume_setup_erupt(plume_ctx* ctx, const PlumeDuct* duct, uint64_t key_base, size_t* added, size_t* removed,
                      double* mass_out, double* sml_out) {
  if (!ctx || !duct || !added || !removed) return PLUME_E_INVALID;
  *added = *removed = 0;
  if (ctx->o.dim != 3 || ctx->nmem != 1 || !(duct->radius > 0) || !(duct->depth > 0) || duct->np < 1) {
    ctx->err = "setup_erupt: single-run 3D contexts, radius, depth > 0, np >= 1";
    return PLUME_E_INVALID;
  }
  // Compute_mass (sph_lib.cc:1024-1040) over the box [-r, r]^2 x [z_top - depth, z_top]
  const double r = duct->radius;
  const double lo[3] = {-r, -r, duct->z_top - duct->depth}, hi[3] = {r, r, duct->z_top};
  double vol = 1.0;
  for (int a = 0; a < 3; a++) vol *= hi[a] - lo[a];
  const double sml = cbrt(vol / duct->np);
  const double mss = duct->rho * vol / duct->np;
  const double s2 = 0.5 * sml;
  int rc = search(ctx);
  if (rc) return rc;
  // Upper bounds of the lattice's axis counts, from the extents alone (one
  // extra point per direction covers the rounding of the repeated steps),
  // checked against the capacity before any host or device memory is
  // taken: a large np makes sml tiny and the lattice huge.
  auto axis_ub = [&](double c0, double a0, double a1) {
    const double up = floor(fmax(a1 - c0 - s2, -sml) / sml) + 2.0;
    const double dn = floor(fmax(c0 - s2 - a0, -sml) / sml) + 2.0;
    return fmax(up, 0.0) + fmax(dn, 0.0);
  };
  const double nz_ub = floor(fmax(hi[2] - s2 - lo[2], -sml) / sml) + 2.0;
  const double ub = axis_ub(duct->x0, -r, r) * axis_ub(duct->y0, -r, r) * fmax(nz_ub, 0.0);
  if (!(sml > 0) || !(ub == ub) || (double)ctx->n_alloc + ub > (double)ctx->cap || ub > (double)INT_MAX) {
    ctx->err = "setup_erupt: the duct lattice (np particles) exceeds the context's capacity";
    return PLUME_E_CAPACITY;
  }
  // the duct lattice (setup_erupt.cc:104-230): axes from the vent axis
  // outward, + side then - side, positions by repeated steps
  auto side = [&](double c0, double a0, double a1, std::vector<double>& out) {
    for (double v = c0 + s2; v <= a1; v += sml) out.push_back(v);
    for (double v = c0 - s2; v >= a0; v -= sml) out.push_back(v);
  };
  std::vector<double> xs, ys, zs, xy;
  side(duct->x0, -r, r, xs);
  side(duct->y0, -r, r, ys);
  for (double z = hi[2] - s2; z >= lo[2]; z -= sml) zs.push_back(z);
  for (double x : xs)
    for (double y : ys)
      if (x * x + y * y <= r * r) {
        xy.push_back(x);
        xy.push_back(y);
      }
  const int npairs = (int)(xy.size() / 2), nz = (int)zs.size();
  const size_t nnew = (size_t)npairs * (size_t)nz;
  if (ctx->n_alloc + nnew > ctx->cap) {
    ctx->err = "setup_erupt exceeds capacity";
    return PLUME_E_CAPACITY;
  }
  cudaStream_t st = ctx->st;
  ScratchFree scratch;
  double *dxy = nullptr, *dz = nullptr;
  unsigned int* drem = nullptr;
  // every scratch buffer is allocated and filled before the removal kernel
  // marks particles dead, so a failure leaves the table untouched
  CK(cudaMalloc(&drem, sizeof(unsigned int)));
  scratch.p[0] = drem;
  if (nnew) {
    CK(cudaMalloc(&dxy, 8 * xy.size()));
    scratch.p[1] = dxy;
    CK(cudaMalloc(&dz, 8 * zs.size()));
    scratch.p[2] = dz;
    CK(cudaMemcpyAsync(dxy, xy.data(), 8 * xy.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dz, zs.data(), 8 * zs.size(), cudaMemcpyHostToDevice, st));
  }
  CK(cudaMemsetAsync(drem, 0, sizeof(unsigned int), st));
  const int n = (int)ctx->n_alloc;
  k_duct_remove<<<nblocks(n ? n : 1), NTHREADS, 0, st>>>(ctx->A, ctx->d_count, r * r, lo[2], hi[2], drem);
  // from here on the table may hold dead rows: the next search compacts them
  const bool had_dead = ctx->has_dead;
  ctx->pending_dead = true;
  ctx->has_dead = true;
  CK(cudaGetLastError());
  ctx->launches++;
  if (nnew) {
    k_duct_fill<<<nblocks(nnew), NTHREADS, 0, st>>>(ctx->d_opt, ctx->A, dxy, npairs, dz, nz, *duct, mss, sml,
                                                   ctx->n_alloc, (unsigned long long)key_base);
    CK(cudaGetLastError());
    ctx->launches++;
  }
  unsigned int nrem = 0;
  CK(cudaMemcpyAsync(&nrem, drem, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (nnew) {
    rc = set_count(ctx, ctx->n_alloc + nnew);
    if (rc) return rc;
  }
  ctx->has_dead = had_dead || nrem != 0;
  *added = nnew;
  *removed = nrem;
  if (mass_out) *mass_out = mss;
  if (sml_out) *sml_out = sml;
  return PLUME_OK;
}

int plume_adapt_step(plume_ctx* ctx, const PlumeAtmosphere* atm, uint64_t key_base, int* adapted,
                     size_t* added) {
  if (!ctx || !atm || !adapted || !added) return PLUME_E_INVALID;
  *adapted = 0;
  *added = 0;
  int a = 0;
  int rc = plume_scan_outside_layer(ctx, &a);
  if (rc) return rc;
  *adapted = a;
  if (!a) return PLUME_OK;
  rc = plume_adapt_domain(ctx);
  if (rc) return rc;
  size_t n1 = 0, n2 = 0;
  rc = plume_add_pressure_ghost(ctx, atm, key_base, &n1);
  if (rc) return rc;
  rc = plume_add_wall_ghost(ctx, atm, key_base + n1, &n2);
  if (rc) return rc;
  *added = n1 + n2;
  if (ctx->nimg) {  // the wall boundary is in use: new ghosts need images
    size_t ni = 0;
    rc = plume_search_bnd_images(ctx, &ni);
    if (rc) return rc;
    rc = plume_apply_bcond(ctx);
    if (rc) return rc;
  }
  return PLUME_OK;
}

int plume_apply_bcond(plume_ctx* ctx) {
  if (!ctx) return PLUME_E_INVALID;
  if (!ctx->nimg) return PLUME_OK;
  int rc = search(ctx);
  if (rc) return rc;
  apply_bc(ctx);
  CK(cudaGetLastError());
  return finish_steps(ctx);
}

// ---------------------------------------------------------------- eruption inlet
int plume_set_inlet(plume_ctx* ctx, const PlumeInlet* in, int reserve_per_step) {
  if (!ctx) return PLUME_E_INVALID;
  if (ctx->inlet_buf) { cudaFree(ctx->inlet_buf); ctx->inlet_buf = nullptr; }
  if (ctx->inlet_colcnt) { cudaFree(ctx->inlet_colcnt); ctx->inlet_colcnt = nullptr; }
  if (ctx->inlet_rowctr) { cudaFree(ctx->inlet_rowctr); ctx->inlet_rowctr = nullptr; }
  ctx->inlet = Inlet{};
  ctx->inlet_reserve = 0;
  if (!in || in->ncol == 0) return PLUME_OK;
  if (ctx->o.dim != 3 || ctx->nmem != 1 || !in->col_xy || !in->col_vel || reserve_per_step < 1 ||
      !(in->spacing > 0)) {
    ctx->err = "inlet: one 3D run, columns with velocities, spacing > 0, reserve >= 1";
    return PLUME_E_INVALID;
  }
  for (size_t c = 0; c < in->ncol; c++)
    if (!(in->col_vel[c] > 0)) {
      ctx->err = "inlet: column velocity must be > 0";
      return PLUME_E_INVALID;
    }
  const size_t nc = in->ncol;
  std::vector<double> h(3 * nc);
  for (size_t c = 0; c < nc; c++) {
    h[2 * c] = in->col_xy[2 * c];
    h[2 * c + 1] = in->col_xy[2 * c + 1];
    h[2 * nc + c] = in->col_vel[c];
  }
  CK(cudaMalloc(&ctx->inlet_buf, 8 * 3 * nc));
  CK(cudaMalloc(&ctx->inlet_colcnt, 8 * nc));
  CK(cudaMalloc(&ctx->inlet_rowctr, sizeof(int)));
  CK(cudaMemcpy(ctx->inlet_buf, h.data(), 8 * 3 * nc, cudaMemcpyHostToDevice));
  std::vector<unsigned long long> cc(nc);
  for (size_t c = 0; c < nc; c++) cc[c] = in->col_count ? in->col_count[c] : 0ull;
  CK(cudaMemcpy(ctx->inlet_colcnt, cc.data(), 8 * nc, cudaMemcpyHostToDevice));
  Inlet& d = ctx->inlet;
  d.xy = ctx->inlet_buf;
  d.vel = ctx->inlet_buf + 2 * nc;
  d.ncol = (int)nc;
  d.bot = in->bot; d.spacing = in->spacing; d.mass = in->mass; d.h = in->h; d.rho = in->rho;
  d.e = in->e; d.p = in->p; d.gam = in->gamma; d.c = in->c; d.Y = in->Y;
  d.key_base = in->key_base;
  ctx->inlet_reserve = reserve_per_step;
  // rows past the live ones are dead (the sort of the next step covers
  // `reserve` of them)
  const size_t from = ctx->n_alloc, to = std::min(ctx->cap, ctx->n_alloc + (size_t)reserve_per_step);
  if (to > from) k_mark_dead<<<nblocks(to - from, 256), 256, 0, ctx->st>>>(ctx->A.bc, from, to);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->st));
  return PLUME_OK;
}

int plume_phase_times(plume_ctx* ctx, float* ms, int n) {
  if (!ctx || !ms) return PLUME_E_INVALID;
  for (int k = 0; k < n && k < NPHASE; k++) ms[k] = ctx->phase_ms[k];
  return PLUME_OK;
}

int plume_launch_count(plume_ctx* ctx, uint64_t* n) {
  if (!ctx || !n) return PLUME_E_INVALID;
  *n = ctx->launches;
  return PLUME_OK;
}

}  // extern "C"
