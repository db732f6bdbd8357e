// sph_kernels.cuh -- the per-step kernels of the particle path.
//
// Particles are stored sorted by fine cell (sub-cells of the reference's
// buckets, row-major with x fastest); cell_start[c] is the first sorted
// index whose cell is >= c, so the particles of cells [c0, c1] of one x-row
// are the index range [cell_start[c0], cell_start[c1 + 1]).  A sweep visits,
// for particle i, the rows of its search box clipped to the 27 buckets
// around its own bucket (search_neighs_consth, neighs.cc:37-211), split at
// bucket boundaries so that "j is in the own bucket" is constant per
// segment.  A candidate j is in the reference's neighbour list of i iff it
// is in the own bucket (neighs.cc:89-92) or inside the list_factor * h_i box
// (neighs.cc:84,128-131), with h_i the smoothing length at the search.
//
// Ensembles: every particle carries its member id; a kernel reads the
// member's grid (Geo), time state and options from per-member tables and
// indexes the cell-start and per-bucket tables from the member's bases, so
// that members never see each other's particles and a member computes what
// it would compute alone.
#pragma once
#include "sph_device.cuh"

namespace plume {

// ---------------------------------------------------------------- segments
// Conservative fine-cell range of [x - R, x + R] on axis a, from the
// particle's bucket index and its FP32 bucket-relative coordinate: every
// cell holding a particle within R is inside the range (the margin covers
// FP32 rounding; exact tests follow in the sweeps), clipped to the 27
// buckets around the particle's bucket and to the grid.  Keeps the range
// arithmetic off the FP64 pipe.
__device__ __forceinline__ void cell_range(const Geo& g, int a, int b, float xr, double R, int& lo, int& hi) {
  const float cwf = (float)g.cw;
  const float icw = 1.0f / cwf;
  const float Rf = (float)R * 1.00001f + 1.0e-3f * cwf;
  const int l = b * g.s + (int)floorf((xr - Rf) * icw);
  const int h = b * g.s + (int)floorf((xr + Rf) * icw);
  lo = max(l, max((b - 1) * g.s, 0));
  hi = min(h, min((b + 2) * g.s - 1, g.G[a] - 1));
}

// Offsets (i's bucket - segment's bucket) * del are passed for the
// bucket-relative FP32 coordinates of the mixed path; the FP64 path works on
// absolute coordinates and gets zero offsets.  CARRY: the segments' bucket
// indices are carried along the loops instead of divided out per row and
// segment (the same segments).
template <int D, typename T, bool CARRY = false, class F>
__device__ __forceinline__ void for_segments(const Geo& g, const uint32_t* __restrict__ cs, const double* xi,
                                             const int* bi, double R, F&& f) {
  if constexpr (D == 1) {
    int lo = cell_axis(g, 0, xi[0] - R, nullptr, nullptr);
    int hi = cell_axis(g, 0, xi[0] + R, nullptr, nullptr);
    f(cs[lo], cs[hi + 1], true, T(0), T(0), T(0));
    return;
  } else {
  int lo[3], hi[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    int l = cell_axis(g, a, xi[a] - R, nullptr, nullptr);
    int h = cell_axis(g, a, xi[a] + R, nullptr, nullptr);
    int bl = (bi[a] - 1) * g.s;
    int bh = (bi[a] + 2) * g.s - 1;
    lo[a] = max(l, max(bl, 0));
    hi[a] = min(h, min(bh, g.G[a] - 1));
  }
  constexpr bool REL = sizeof(T) == 4;
  const T delT = T(g.del);
  if constexpr (!CARRY) {
  for (int cz = lo[2]; cz <= hi[2]; cz++) {
    int bz = cz / g.s;
    T oz = REL ? T(bi[2] - bz) * delT : T(0);
    for (int cy = lo[1]; cy <= hi[1]; cy++) {
      int by = cy / g.s;
      T oy = REL ? T(bi[1] - by) * delT : T(0);
      size_t rowbase = ((size_t)cz * g.G[1] + cy) * (size_t)g.G[0];
      int cx = lo[0];
      while (cx <= hi[0]) {
        int bx = cx / g.s;
        int e = min(hi[0], bx * g.s + g.s - 1);
        bool own = (bx == bi[0]) && (by == bi[1]) && (bz == bi[2]);
        f(cs[rowbase + cx], cs[rowbase + e + 1], own, REL ? T(bi[0] - bx) * delT : T(0), oy, oz);
        cx = e + 1;
      }
    }
  }
  } else {
  // bucket indices carried along the loops (one division per axis): a
  // segment ends at its bucket's last cell, so the next one starts a bucket on
  const int bx0 = lo[0] / g.s, by0 = lo[1] / g.s;
  int bz = lo[2] / g.s, rz = lo[2] - bz * g.s;
  for (int cz = lo[2]; cz <= hi[2]; cz++) {
    T oz = REL ? T(bi[2] - bz) * delT : T(0);
    int by = by0, ry = lo[1] - by0 * g.s;
    for (int cy = lo[1]; cy <= hi[1]; cy++) {
      T oy = REL ? T(bi[1] - by) * delT : T(0);
      size_t rowbase = ((size_t)cz * g.G[1] + cy) * (size_t)g.G[0];
      int cx = lo[0], bx = bx0;
      while (cx <= hi[0]) {
        int e = min(hi[0], bx * g.s + g.s - 1);
        bool own = (bx == bi[0]) && (by == bi[1]) && (bz == bi[2]);
        f(cs[rowbase + cx], cs[rowbase + e + 1], own, REL ? T(bi[0] - bx) * delT : T(0), oy, oz);
        cx = e + 1;
        bx++;
      }
      if (++ry == g.s) { ry = 0; by++; }
    }
    if (++rz == g.s) { rz = 0; bz++; }
  }
  }
  }
}

// The candidates of a particle's stored neighbour list (search_neighs_consth,
// neighs.cc:84-131: its own bucket, and the particles of the 26 others
// inside the list box), walked as two regions: A, the rows within RA (the
// list box, or less when the caller's reach is shorter) clipped to the 27
// buckets, then B, the fine cells of the own bucket outside A's cells.  Every
// candidate of the list inside RA comes once; f gets own = true for B.
template <typename T, class F>
__device__ __forceinline__ void walk_list_region(const Geo& g, const uint32_t* __restrict__ cs, const double* xi,
                                                 const int* bi, double RA, F&& f) {
  for_segments<3, T>(g, cs, xi, bi, RA, f);
  int lo[3], hi[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const int l = cell_axis(g, a, xi[a] - RA, nullptr, nullptr);
    const int h = cell_axis(g, a, xi[a] + RA, nullptr, nullptr);
    lo[a] = max(l, max((bi[a] - 1) * g.s, 0));
    hi[a] = min(h, min((bi[a] + 2) * g.s - 1, g.G[a] - 1));
  }
  const int b0 = bi[0] * g.s, b1 = b0 + g.s - 1;
  for (int cz = bi[2] * g.s; cz < (bi[2] + 1) * g.s; cz++)
    for (int cy = bi[1] * g.s; cy < (bi[1] + 1) * g.s; cy++) {
      const size_t rowbase = ((size_t)cz * g.G[1] + cy) * (size_t)g.G[0];
      if (cz >= lo[2] && cz <= hi[2] && cy >= lo[1] && cy <= hi[1]) {
        // the parts of the own bucket's x-run outside A's cells
        if (lo[0] > b0) f(cs[rowbase + b0], cs[rowbase + min(lo[0] - 1, b1) + 1], true, T(0), T(0), T(0));
        if (hi[0] < b1) f(cs[rowbase + max(hi[0] + 1, b0)], cs[rowbase + b1 + 1], true, T(0), T(0), T(0));
      } else {
        f(cs[rowbase + b0], cs[rowbase + b1 + 1], true, T(0), T(0), T(0));
      }
    }
}

template <int D>
__device__ __forceinline__ void bucket_coords(const Geo& g, int b, int* bi) {
  if (D == 1) {
    bi[0] = b; bi[1] = 0; bi[2] = 0;
  } else {
    bi[0] = b % g.nb[0];
    bi[1] = (b / g.nb[0]) % g.nb[1];
    bi[2] = b / (g.nb[0] * g.nb[1]);
  }
}

// position of particle j in the sweep's arithmetic: absolute (FP64 path) or
// bucket-relative (mixed path)
template <int D, typename T>
struct Pos;
template <int D>
struct Pos<D, double> {
  __device__ __forceinline__ static void load(const Dev& A, const Work&, int j, double* x) {
    x[0] = A.x[j];
    if (D == 3) { x[1] = A.y[j]; x[2] = A.z[j]; }
  }
};
template <int D>
struct Pos<D, float> {
  __device__ __forceinline__ static void load(const Dev&, const Work& W, int j, float* x) {
    x[0] = W.xr[j];
    if (D == 3) { x[1] = W.yr[j]; x[2] = W.zr[j]; }
  }
};

// dx = x_i - x_j in the sweep's arithmetic.  3D mixed: bucket-relative FP32
// coordinates plus the segment's bucket offset; 1D mixed (every cell is its
// own bucket): the FP64 difference rounded to FP32; FP64: absolute.
template <int D, typename T>
__device__ __forceinline__ void pair_dx(const T* xsh, const double* xi, const Dev& A, const Work& W, uint32_t j,
                                        T* dx) {
  if constexpr (D == 1 && sizeof(T) == 4) {
    dx[0] = (T)(xi[0] - A.x[j]);
  } else {
    T xj[3];
    Pos<D, T>::load(A, W, j, xj);
#pragma unroll
    for (int k = 0; k < D; k++) dx[k] = xsh[k] - xj[k];
  }
}

template <int D, typename T>
__device__ __forceinline__ bool in_box(const T* dx, T r) {
#pragma unroll
  for (int k = 0; k < D; k++)
    if (fabs(dx[k]) > r) return false;
  return true;
}

// ---------------------------------------------------------------- adaptive
// adaptive_sml (neighs.cc:479-693, ADAPTIVE_SML 1): up to num_loop fixed-point
// iterations h <- eta * (m / rho*)^(1/D), rho* = sum m_j W(dx / 2h, 2h)
// Runs on the steps with hstep % interval == 0 unless forced.
// hit / nit (adjoint recording, null otherwise): the iterates h_0..h_K in
// rows of nrow and the iteration count K of every particle.
template <int D, typename T>
__global__ void k_adaptive(Opt o, const Geo* __restrict__ geo, Dev A, Work W, const uint32_t* __restrict__ cs_all,
                           const int* __restrict__ d_count, TimeState* ts_all, const int* __restrict__ hstep,
                           int force, double* __restrict__ hit = nullptr, uint8_t* __restrict__ nit = nullptr,
                           int nrow = 0) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count) return;
  if (!force && (*hstep % o.interval) != 0) return;
  if (!need_neigh(A.bc[i])) return;
  const int m = A.mem[i];
  TimeState* ts = ts_all + m;
  if (!ts->active) return;
  const Geo g = geo[m];
  const uint32_t* cs = cs_all + g.cell_base;
  double xi[3] = {A.x[i], D == 3 ? A.y[i] : 0.0, D == 3 ? A.z[i] : 0.0};
  int bi[3];
  bucket_coords<D>(g, A.bkt[i], bi);
  T xs[3];
  Pos<D, T>::load(A, W, i, xs);
  const T Lb = T(o.list_factor * W.hlist[i]);
  const double mi = A.mass[i];
  double hcur = A.h[i];
  int done = 0;
  for (int loop = 0; loop < o.num_loop; loop++) {
    double H_old = hcur;
    if (hit) hit[(size_t)loop * nrow + i] = H_old;
    done = loop + 1;
    double H_star_d = H_old * o.c_smooth;
    T H_star = T(H_star_d);
    T supp = T(o.cutoff2) * H_star;
    Acc<T> rho_star;
    double R = fmin(o.cutoff2, o.ksupport) * H_star_d * (1.0 + 1e-10);
    auto visit = [&](uint32_t j0, uint32_t j1, bool own, T ox, T oy, T oz) {
      T xsh[3] = {xs[0] + ox, D == 3 ? xs[1] + oy : T(0), D == 3 ? xs[2] + oz : T(0)};
      for (uint32_t j = j0; j < j1; j++) {
        if (!contr_dens(A.bc[j], o.pgc)) continue;
        T dx[3], si[3];
        pair_dx<D, T>(xsh, xi, A, W, j, dx);
#pragma unroll
        for (int k = 0; k < D; k++) si[k] = dx[k] / H_star;
        if (!own && !in_box<D, T>(dx, Lb)) continue;
        if (!in_box<D, T>(dx, supp)) continue;
        T mj = T(A.mass[j]);
        T wght = kw<D, T>(o.kernel, si, H_star);
        rho_star.add(wght * mj);
      }
    };
    // 3D: the list's own bucket plus its list box (the reach beyond the
    // list box holds no listed candidate)
    if constexpr (D == 3)
      walk_list_region<T>(g, cs, xi, bi, fmin(R, o.list_factor * W.hlist[i] * (1.0 + 1e-6)), visit);
    else
      for_segments<D, T>(g, cs, xi, bi, R, visit);
    double rs = (double)rho_star.get();
    double H_new = (D == 3) ? o.eta * cbrt(mi / rs) : o.eta * (mi / rs);
    hcur = 1.0 * H_new;
    if (!(H_new > 0) || !isfinite(H_new)) {
      set_status(ts, 4);
      break;
    }
    double err = fabs((H_new - H_old) / H_old);
    if (err < o.thresh) break;
  }
  if (hit) {
    hit[(size_t)done * nrow + i] = hcur;
    nit[i] = (uint8_t)done;
  }
  A.h[i] = hcur;
}

// ---------------------------------------------------------------- momentum
// mom_engr_update, USE_GSPH == 0 (mom_engr_update.cc:96-354)
template <int D, typename T>
__global__ void k_momentum(Opt o, const Geo* __restrict__ geo, Dev A, Work W, const uint32_t* __restrict__ cs_all,
                           const double* __restrict__ hmax_all, const int* __restrict__ d_count,
                           TimeState* ts_all) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count) return;
  if (!need_neigh(A.bc[i])) return;
  const int m = A.mem[i];
  TimeState* ts = ts_all + m;
  if (!ts->active) return;
  const Geo g = geo[m];
  const uint32_t* cs = cs_all + g.cell_base;
  const double* hmax = hmax_all + g.bucket_base;
  const double dt = ts->dtime;
  double xi[3] = {A.x[i], D == 3 ? A.y[i] : 0.0, D == 3 ? A.z[i] : 0.0};
  int bi[3];
  const int b = A.bkt[i];
  bucket_coords<D>(g, b, bi);
  T xs[3];
  Pos<D, T>::load(A, W, i, xs);
  const double hi_d = A.h[i];
  const double rho_i_d = A.rho[i];
  if (!(rho_i_d > 0)) {
    set_status(ts, 4);
    return;
  }
  const T hi = T(hi_d);
  const T supp = T(o.cutoff2) * hi;
  const T Lb = T(o.list_factor * W.hlist[i]);
  const T rhoi = T(rho_i_d);
  const T Vi = T(1.0) / rhoi;
  const T pvsqi = T(A.p[i]) * Vi * Vi;
  const T ci = T(A.c[i]);
  const T tempi = T(A.T[i]);
  const T Cp_i = T(A.cp[i]);
  T veli[3];
  if (o.lans) {
    veli[0] = T(A.vsx[i]);
    if (D == 3) { veli[1] = T(A.vsy[i]); veli[2] = T(A.vsz[i]); }
  } else {
    veli[0] = T(A.vx[i]);
    if (D == 3) { veli[1] = T(A.vy[i]); veli[2] = T(A.vz[i]); }
  }
  Acc<T> rhs_v[3], rhs_e;
  const double hm = hmax[D == 3 ? b : 0];
  const double R = fmin(o.cutoff2 * hi_d, o.ksupport * 0.5 * (hi_d + hm)) * (1.0 + 1e-10);
  const bool lans = o.lans != 0;
  for_segments<D, T>(g, cs, xi, bi, R, [&](uint32_t j0, uint32_t j1, bool own, T ox, T oy, T oz) {
    T xsh[3] = {xs[0] + ox, D == 3 ? xs[1] + oy : T(0), D == 3 ? xs[2] + oz : T(0)};
    for (uint32_t j = j0; j < j1; j++) {
      if (j == (uint32_t)i) continue;
      T dx[3];
      pair_dx<D, T>(xsh, xi, A, W, j, dx);
      if (!own && !in_box<D, T>(dx, Lb)) continue;
      if (!in_box<D, T>(dx, supp)) continue;
      const T hj = T(A.h[j]);
      const T h = T(0.5) * (hi + hj);
      T si[3], dist_sq = 0;
#pragma unroll
      for (int k = 0; k < D; k++) {
        si[k] = dx[k] / h;
        dist_sq += dx[k] * dx[k];
      }
      const T mj = T(A.mass[j]);
      const T pressj = T(A.p[j]);
      const T rhoj = T(A.rho[j]);
      const T Vj = T(1.0) / rhoj;
      T velij[3];
      if (lans) {
        velij[0] = veli[0] - T(A.vsx[j]);
        if (D == 3) { velij[1] = veli[1] - T(A.vsy[j]); velij[2] = veli[2] - T(A.vsz[j]); }
      } else {
        velij[0] = veli[0] - T(A.vx[j]);
        if (D == 3) { velij[1] = veli[1] - T(A.vy[j]); velij[2] = veli[2] - T(A.vz[j]); }
      }
      const T rhoab = T(0.5) * (rhoi + rhoj);
      const T sndspdab = T(0.5) * (ci + T(A.c[j]));
      // art_vis
      T vrab = 0;
#pragma unroll
      for (int k = 0; k < D; k++) vrab += dx[k] * velij[k];
      const T miuab = h * vrab / (dist_sq + T(o.ata) * h * h);
      T vis = 0;
      if (vrab < 0) vis = (T(o.beta) * miuab - T(o.alpha) * sndspdab) * miuab / rhoab;
      T dotv = 0;
      if (lans) {
#pragma unroll
        for (int k = 0; k < D; k++) dotv += velij[k] * velij[k];
        vis -= T(EPS_HALF) * dotv * Vj;
      }
      const T mpvsqij = mj * (pressj * Vj * Vj + pvsqi + vis);
      T dwdx[3];
      kdw<D, T>(o.kernel, si, h, dwdx);
      T heat_tran = 0;
      if (lans) {
        const T Cp_ij = T(0.5) * (T(A.cp[j]) + Cp_i);
        // SPH_epsilon_heat_conductivity(Cp_ij, dx, velij, rhoab, hab=h, sndspdab)
        T dotvr = 0, dotrr = 0;
#pragma unroll
        for (int k = 0; k < D; k++) dotvr += fabs(velij[k] * dx[k]);
        T kij = 0;
        if (dotvr != T(0)) {
#pragma unroll
          for (int k = 0; k < D; k++) dotrr += dx[k] * dx[k];
          T kab;
          if (D == 3)
            kab = T(10.0) * T(EPS_HALF) * Cp_ij * dotrr * dotv / (T(PRANDTL) * dotvr);
          else
            kab = 0;
          kij = kab / (h * sndspdab);
        }
        // compute_F(dwdx, dx)
        T W_r = 0, r_sq = 0, Fij = 0;
#pragma unroll
        for (int k = 0; k < D; k++) W_r += dwdx[k] * dx[k];
        if (W_r != T(0)) {
#pragma unroll
          for (int k = 0; k < D; k++) r_sq += dx[k] * dx[k];
          Fij = W_r / r_sq;
        }
        heat_tran = mj * Vj * Vi * kij * (tempi - T(A.T[j])) * Fij;
      }
#pragma unroll
      for (int k = 0; k < D; k++) rhs_v[k].sub(mpvsqij * dwdx[k]);
      T deltae = 0;
#pragma unroll
      for (int k = 0; k < D; k++) deltae += T(0.5) * (mpvsqij * dwdx[k]) * velij[k];
      rhs_e.add(deltae + heat_tran);
    }
  });
  const double grav = -o.g;
  double vi[3] = {A.vx[i], D == 3 ? A.vy[i] : 0.0, D == 3 ? A.vz[i] : 0.0};
  double unew[3];
#pragma unroll
  for (int k = 0; k < D; k++) unew[k] = vi[k] + dt * (double)rhs_v[k].get();
  unew[D - 1] += dt * grav;
  W.nv0[i] = unew[0];
  if (D == 3) { W.nv1[i] = unew[1]; W.nv2[i] = unew[2]; }
  W.ne[i] = A.e[i] + dt * ((double)rhs_e.get() + (double)veli[D - 1] * grav);
}

// commit loop of mom_engr_update.cc:412-432
template <int D>
__global__ void k_commit_mom(const Opt* __restrict__ mopt, Dev A, Work W, const int* __restrict__ d_count,
                             const TimeState* __restrict__ ts_all) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count) return;
  if (!need_neigh(A.bc[i])) return;
  const int m = A.mem[i];
  if (!ts_all[m].active) return;
  const Opt& o = mopt[m];
  A.vx[i] = W.nv0[i];
  if (D == 3) { A.vy[i] = W.nv1[i]; A.vz[i] = W.nv2[i]; }
  double e = W.ne[i];
  A.e[i] = e;
  double gam, p, c, T, cp = A.cp[i];
  eos(o, A.rho[i], A.Y[i], e, gam, p, c, T, cp, o.lans != 0);
  A.gam[i] = gam; A.p[i] = p; A.c[i] = c; A.T[i] = T; A.cp[i] = cp;
}

// ---------------------------------------------------------------- density
// smooth_density (density_massfrac.cc:64-333), DENSITY_UPDATE_SML 11,
// DENSITY_UPDATE_SPH 11, optional normalised energy smoothing
template <int D, typename T>
__global__ void k_density(Opt o, const Geo* __restrict__ geo, Dev A, Work W, const uint32_t* __restrict__ cs_all,
                          const double* __restrict__ hmax_all, const int* __restrict__ d_count,
                          TimeState* ts_all) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count) return;
  if (!need_neigh(A.bc[i])) return;
  const int m = A.mem[i];
  TimeState* ts = ts_all + m;
  if (!ts->active) return;
  const Geo g = geo[m];
  const uint32_t* cs = cs_all + g.cell_base;
  const double* hmax = hmax_all + g.bucket_base;
  double xi[3] = {A.x[i], D == 3 ? A.y[i] : 0.0, D == 3 ? A.z[i] : 0.0};
  int bi[3];
  const int b = A.bkt[i];
  bucket_coords<D>(g, b, bi);
  T xs[3];
  Pos<D, T>::load(A, W, i, xs);
  const double hi_d = A.h[i];
  const T hi = T(hi_d);
  const T supp = T(o.cutoff2) * hi;
  const T Lb = T(o.list_factor * W.hlist[i]);
  Acc<T> rho1, rho2, wnorm_e, engr;
  const double hm = hmax[D == 3 ? b : 0];
  const double R = fmin(o.cutoff2 * hi_d, o.ksupport * 0.5 * (hi_d + hm)) * (1.0 + 1e-10);
  const bool esm = o.esmooth != 0;
  for_segments<D, T>(g, cs, xi, bi, R, [&](uint32_t j0, uint32_t j1, bool own, T ox, T oy, T oz) {
    T xsh[3] = {xs[0] + ox, D == 3 ? xs[1] + oy : T(0), D == 3 ? xs[2] + oz : T(0)};
    for (uint32_t j = j0; j < j1; j++) {
      const uint8_t bcj = A.bc[j];
      if (!contr_dens(bcj, o.pgc)) continue;
      const uint8_t ph = A.phase[j];
      if (ph != 1 && ph != 2) continue;
      T ds[3];
      pair_dx<D, T>(xsh, xi, A, W, j, ds);
      if (!own && !in_box<D, T>(ds, Lb)) continue;
      if (!in_box<D, T>(ds, supp)) continue;
      const T mj = T(A.mass[j]);
      const T hh = T(0.5) * (hi + T(A.h[j]));
      T s[3];
#pragma unroll
      for (int k = 0; k < D; k++) s[k] = ds[k] / hh;
      if (esm) {
        const T rhoj = T(A.rho[j]);
        T s_e[3];
#pragma unroll
        for (int k = 0; k < D; k++) s_e[k] = T(E_SMOOTH) * ds[k] / hh;
        const T wm_e = kw<D, T>(o.kernel, s_e, hh / T(E_SMOOTH)) * mj;
        wnorm_e.add(wm_e / rhoj);
        engr.add(wm_e * T(A.e[j]) / rhoj);
      }
      const T wm = kw<D, T>(o.kernel, s, hh) * mj;
      if (ph == 1)
        rho1.add(wm);
      else
        rho2.add(wm);
    }
  });
  if (esm) {
    double wn = (double)wnorm_e.get();
    if (!(wn > 0)) {
      set_status(ts, 4);
      return;
    }
    W.nE[i] = (double)engr.get() / wn;
  }
  double density = 0.0;
  density += (double)rho1.get();
  density += (double)rho2.get();
  if (!(density > 0)) {
    set_status(ts, (density != density) ? 3 : 4);
    return;
  }
  W.nrho[i] = density;
  W.nY[i] = (double)rho2.get() / density;
}

// commit loop of density_massfrac.cc:337-352
template <int D>
__global__ void k_commit_dens(const Opt* __restrict__ mopt, Dev A, Work W, const int* __restrict__ d_count,
                              const TimeState* __restrict__ ts_all) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count) return;
  if (!need_neigh(A.bc[i])) return;
  const int m = A.mem[i];
  if (!ts_all[m].active) return;
  const Opt& o = mopt[m];
  double Y = W.nY[i];
  A.Y[i] = Y;
  if (Y >= MSFRC_TH && A.inv[i] != 2) A.inv[i] = 2;
  double rho = W.nrho[i];
  A.rho[i] = rho;
  double e = A.e[i];
  if (o.esmooth) {
    e = W.nE[i];
    A.e[i] = e;
  }
  double gam, p, c, T, cp = A.cp[i];
  eos(o, rho, Y, e, gam, p, c, T, cp, o.lans != 0);
  A.gam[i] = gam; A.p[i] = p; A.c[i] = c; A.T[i] = T; A.cp[i] = cp;
}

// ---------------------------------------------------------------- velocity
// smooth_velocity (smooth_velocity.cc:25-165), HAVE_TURBULENCE_LANS 1
template <int D, typename T>
__global__ void k_velocity(Opt o, const Geo* __restrict__ geo, Dev A, Work W, const uint32_t* __restrict__ cs_all,
                           const int* __restrict__ d_count, TimeState* ts_all) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count) return;
  if (!need_neigh(A.bc[i])) return;
  const int m = A.mem[i];
  TimeState* ts = ts_all + m;
  if (!ts->active) return;
  const Geo g = geo[m];
  const uint32_t* cs = cs_all + g.cell_base;
  double xi[3] = {A.x[i], D == 3 ? A.y[i] : 0.0, D == 3 ? A.z[i] : 0.0};
  int bi[3];
  bucket_coords<D>(g, A.bkt[i], bi);
  T xs[3];
  Pos<D, T>::load(A, W, i, xs);
  const double hi_d = A.h[i];
  const T hi = T(hi_d);
  const T supp = T(o.cutoff2) * hi;
  const T Lb = T(o.list_factor * W.hlist[i]);
  const double vi_d[3] = {A.vx[i], D == 3 ? A.vy[i] : 0.0, D == 3 ? A.vz[i] : 0.0};
  const T vi[3] = {T(vi_d[0]), T(vi_d[1]), T(vi_d[2])};
  Acc<T> dv[3], wnorm;
  const double R = fmin(o.cutoff2, o.ksupport) * hi_d * (1.0 + 1e-10);
  for_segments<D, T>(g, cs, xi, bi, R, [&](uint32_t j0, uint32_t j1, bool own, T ox, T oy, T oz) {
    T xsh[3] = {xs[0] + ox, D == 3 ? xs[1] + oy : T(0), D == 3 ? xs[2] + oz : T(0)};
    for (uint32_t j = j0; j < j1; j++) {
      if (!contr_vel_smooth(A.bc[j])) continue;
      T ds[3];
      pair_dx<D, T>(xsh, xi, A, W, j, ds);
      if (!own && !in_box<D, T>(ds, Lb)) continue;
      if (!in_box<D, T>(ds, supp)) continue;
      const T rhoj = T(A.rho[j]);
      const T mj = T(A.mass[j]);
      T s[3];
#pragma unroll
      for (int k = 0; k < D; k++) s[k] = ds[k] / hi;
      const T wght = kw<D, T>(o.kernel, s, hi);
      const T mvw = wght * mj / rhoj;
      dv[0].add(mvw * (T(A.vx[j]) - vi[0]));
      if (D == 3) {
        dv[1].add(mvw * (T(A.vy[j]) - vi[1]));
        dv[2].add(mvw * (T(A.vz[j]) - vi[2]));
      }
      wnorm.add(mvw);
    }
  });
  double wn = (double)wnorm.get();
  if (!(wn > 0)) {
    set_status(ts, 4);
    return;
  }
  A.vsx[i] = vi_d[0] + (double)dv[0].get() / wn;
  if (D == 3) {
    A.vsy[i] = vi_d[1] + (double)dv[1].get() / wn;
    A.vsz[i] = vi_d[2] + (double)dv[2].get() / wn;
  }
}

// ---------------------------------------------------------------- position
// update_pos (update_pos.cc:34-168) and the deletions of
// update_particles_in_bucket (update_pos.cc:171-463, serial case)
template <int D>
__global__ void k_update_pos(const Opt* __restrict__ mopt, const Geo* __restrict__ geo, Dev A,
                             const uint8_t* __restrict__ bflags_all, const int8_t* __restrict__ bface_all,
                             const int* __restrict__ d_count, TimeState* ts_all) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *d_count) return;
  const int m = A.mem[i];
  TimeState* ts = ts_all + m;
  if (!ts->active) return;
  const Opt& o = mopt[m];
  const Geo g = geo[m];
  const uint8_t* bflags = bflags_all ? bflags_all + g.bucket_base : nullptr;
  const int8_t* bface = bface_all ? bface_all + 6 * (size_t)g.bucket_base : nullptr;
  uint8_t bc = A.bc[i];
  const double dt = ts->dtime;
  double pos[3] = {A.x[i], D == 3 ? A.y[i] : 0.0, D == 3 ? A.z[i] : 0.0};
  bool moved = false;
  if (is_real(bc)) {
    double v[3];
    if (o.lans) {
      v[0] = A.vsx[i];
      if (D == 3) { v[1] = A.vsy[i]; v[2] = A.vsz[i]; }
    } else {
      v[0] = A.vx[i];
      if (D == 3) { v[1] = A.vy[i]; v[2] = A.vz[i]; }
    }
#pragma unroll
    for (int k = 0; k < D; k++) pos[k] = __dadd_rn(pos[k], __dmul_rn(dt, v[k]));
    moved = true;
  } else if (bc == 0 && ts->erupt) {
    double v[3] = {A.vx[i], D == 3 ? A.vy[i] : 0.0, D == 3 ? A.vz[i] : 0.0};
#pragma unroll
    for (int k = 0; k < D; k++) pos[k] = __dadd_rn(pos[k], __dmul_rn(dt, v[k]));
    moved = true;
    if (D == 3 && pos[2] >= o.vent_z) {
      bc = 100;  // erupt_turn_real
      A.bc[i] = 100;
      A.h[i] = 1.0 * o.sml2;
      A.inv[i] = 2;
    }
  }
  if (!moved) return;
  A.x[i] = pos[0];
  if (D == 3) { A.y[i] = pos[1]; A.z[i] = pos[2]; }
  if (D == 1) return;
  const int ob = A.bkt[i];
  const uint8_t of = bflags ? bflags[ob] : 0;
  if (of & 0x4) return;  // inactive bucket
  if (is_real(bc) && (of & 0x2) && bface) {
    const int8_t* fi = bface + 6 * ob;
    bool los = false;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      if (fi[2 * a] == -1) {
        if ((pos[a] - g.lo[a]) < -TINY_D) los = true;
      } else if (fi[2 * a + 1] == 1) {
        if ((pos[a] - g.hi[a]) > TINY_D) los = true;
      }
    }
    if (los) {
      A.bc[i] = BC_DEAD;
      atomicAdd(&ts->n_lost, 1ull);
      return;
    }
  }
  bool out = false, o1, o2, o3;
  int bx = bucket_axis(pos[0], g.mind[0], g.del, g.idel, g.nb[0], &o1);
  int by = bucket_axis(pos[1], g.mind[1], g.del, g.idel, g.nb[1], &o2);
  int bz = bucket_axis(pos[2], g.mind[2], g.del, g.idel, g.nb[2], &o3);
  out = o1 || o2 || o3;
  if (out) {
    set_status(ts, 6);
    return;
  }
  int nb = (bz * g.nb[1] + by) * g.nb[0] + bx;
  if (nb != ob && bflags && (bflags[nb] & 0x1)) {
    A.bc[i] = BC_DEAD;
    atomicAdd(&ts->n_lost, 1ull);
  }
}

}  // namespace plume
