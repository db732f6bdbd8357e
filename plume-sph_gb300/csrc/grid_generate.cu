// grid_generate.cu -- the bucket grid of the reference's preprocessor
// (src/preproc/preprocess.cc:68-177, :386-464, flat ground) on the device.
//
// The preprocessor pads the original domain [lo, hi] by EXT_DOM_COF =
// EXT_DOM_COF_BOT = 1.5 buckets of edge del = PARTICLE_DENSITY * h0 (8 in
// 3D, constant.h:132-136), rounds the bucket counts up, and types every
// bucket from the position of its six faces against the original domain
// (determine_face_type: -1 below, +1 above, 0 inside or on the boundary).
// One thread per bucket computes the same face indices from the same FP64
// corner expressions (mindom + i * del, mindom + (i + 1) * del) and writes
// the PlumeGrid flags the step reads:
//   - a bucket straddling the ground (bottom face below, top face not) is
//     MIXED whatever its other faces say (preprocess.cc:462-463);
//   - else a bucket wholly outside on some axis is absorbing, UNDERGROUND
//     when wholly below the ground, else PRESS_BC (:423-429), and the
//     explicit type bit is set with it;
//   - else a bucket straddling a side or the top is MIXED (:431-432);
//   - else it is OVERGROUND (no flag).
// The hash keys and process ids of the preprocessor are not produced: the
// device addresses buckets by their linear index.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "../../include/plume_gpu.h"

namespace {

__device__ __forceinline__ int8_t face_type(double crd, double hi, double lo) {
  return crd < lo ? -1 : (crd > hi ? 1 : 0);
}

struct GridGeom {
  double mind[3], lo[3], hi[3], del;
  int nb[3];
};

__global__ void k_grid_generate(GridGeom g, uint8_t* __restrict__ flags, int8_t* __restrict__ face, size_t nbk) {
  for (size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x; b < nbk; b += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(b % (size_t)g.nb[0]);
    const int j = (int)((b / (size_t)g.nb[0]) % (size_t)g.nb[1]);
    const int k = (int)(b / ((size_t)g.nb[0] * (size_t)g.nb[1]));
    const int ijk[3] = {i, j, k};
    int8_t bt[6];
    int flag[3];
    for (int a = 0; a < 3; a++) {
      const double c0 = g.mind[a] + ijk[a] * g.del;
      const double c1 = g.mind[a] + (ijk[a] + 1) * g.del;
      bt[2 * a] = face_type(c0, g.hi[a], g.lo[a]);
      bt[2 * a + 1] = face_type(c1, g.hi[a], g.lo[a]);
      flag[a] = abs(bt[2 * a] + bt[2 * a + 1]);
    }
    uint8_t f = 0;
    if (bt[4] == -1 && bt[5] == 0)
      f = PLUME_BUCKET_MIXED;
    else if (flag[0] == 2 || flag[1] == 2 || flag[2] == 2)
      f = PLUME_BUCKET_ABSORBING |
          ((bt[4] == -1 && bt[5] == -1) ? PLUME_BUCKET_UNDERGROUND : PLUME_BUCKET_PRESS_BC);
    else if (flag[0] == 1 || flag[1] == 1 || flag[2] == 1)
      f = PLUME_BUCKET_MIXED;
    flags[b] = f;
    for (int q = 0; q < 6; q++) face[6 * b + q] = bt[q];
  }
}

}  // namespace

extern "C" int plume_grid_generate(const double lo[3], const double hi[3], double h0, int subcells,
                                   PlumeGrid* grid, uint8_t* flags, int8_t* face_index, size_t cap,
                                   size_t* nbk_out) {
  if (!lo || !hi || !grid || !nbk_out || !(h0 > 0) || subcells < 1) return PLUME_E_INVALID;
  GridGeom g{};
  g.del = 8.0 * h0;  // PARTICLE_DENSITY * smoothing length
  size_t nbk = 1;
  for (int a = 0; a < 3; a++) {
    if (!(hi[a] > lo[a])) return PLUME_E_INVALID;
    g.lo[a] = lo[a];
    g.hi[a] = hi[a];
    g.mind[a] = lo[a] - 1.5 * g.del;
    const double maxd = hi[a] + 1.5 * g.del;
    const double n = std::ceil((maxd - g.mind[a]) / g.del);
    if (!(n >= 1) || n > 1.0e6) return PLUME_E_INVALID;
    g.nb[a] = (int)n;
    nbk *= (size_t)g.nb[a];
  }
  *nbk_out = nbk;
  for (int a = 0; a < 3; a++) {
    grid->mindom[a] = g.mind[a];
    grid->nb[a] = g.nb[a];
    grid->domain_lo[a] = lo[a];
    grid->domain_hi[a] = hi[a];
  }
  grid->del = g.del;
  grid->subcells = subcells;
  if (!flags || !face_index) return PLUME_OK;  // sizing call
  if (nbk > cap) return PLUME_E_CAPACITY;
  uint8_t* dflags = nullptr;
  int8_t* dface = nullptr;
  int rc = PLUME_OK;
  if (cudaMalloc(&dflags, nbk) != cudaSuccess || cudaMalloc(&dface, 6 * nbk) != cudaSuccess) {
    rc = PLUME_E_CUDA;
  } else {
    const int threads = 256;
    const size_t want = (nbk + threads - 1) / threads;
    const int blocks = (int)(want < 152 * 8 ? want : 152 * 8);
    k_grid_generate<<<blocks, threads>>>(g, dflags, dface, nbk);
    if (cudaGetLastError() != cudaSuccess || cudaMemcpy(flags, dflags, nbk, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(face_index, dface, 6 * nbk, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = PLUME_E_CUDA;
  }
  if (dflags) cudaFree(dflags);
  if (dface) cudaFree(dface);
  if (rc == PLUME_OK) {
    grid->flags = flags;
    grid->face_index = face_index;
  }
  return rc;
}
