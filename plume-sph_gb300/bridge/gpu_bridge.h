// gpu_bridge.h -- the reference-side binding of the GB300 particle step.
//
// A Plume-SPH build adds gpu_bridge.cc to src/plume/ and links
// libplume_gpu.so; main.cc then hands its particle table to the device
// through the C ABI of plume_gpu.h instead of calling the hot functions of
// particler.h (timestep, search_neighs_consth, adaptive_sml,
// mom_engr_update, smooth_density, smooth_velocity, update_pos,
// update_particles_in_bucket: main.cc:217-408).
//
// The bridge packs the THashTable of Particle objects (datstr/particle.h:
// 27-140) into the structure-of-arrays PlumeSoA, keyed by the row of each
// Particle in `rows`, and writes the device's results back into the same
// objects.  Rows the device deleted leave the table; rows it created (the
// device inlet or ghost layers) become new Particle objects.
#ifndef PLUME_GPU_BRIDGE_H
#define PLUME_GPU_BRIDGE_H

#include <cstdint>
#include <vector>

#include "plume_gpu.h"

class THashTable;
class Particle;

struct GpuBridge {
  plume_ctx *ctx = nullptr;
  std::vector<Particle *> rows;  // 64-bit key of a row = its index here
  std::vector<uint64_t> key;
  std::vector<double> f[19];     // x y z vx vy vz vsx vsy vsz m h rho e p Y gamma c T cp
  std::vector<uint8_t> phase, bc, inv;
  int myid = 0;

  // the SoA view of the bridge's arrays
  PlumeSoA soa();
  // every particle of the table (any bc_type) into the arrays; returns n
  size_t pack(THashTable *P);
  // the rows of the arrays back into the table: rows [0, n) in device order
  // (the first n of the arrays); rows of known keys update their Particle,
  // keys beyond the packed rows create Particles; packed rows that are
  // absent were deleted and leave the table
  void unpack_rows(THashTable *P, size_t n);
  // plume_upload of the packed table
  int upload();
  // plume_download into the arrays (room for `cap` rows), then unpack_rows
  int download(THashTable *P, size_t cap);
};

#endif
