// gpu_bridge.cc -- pack the reference's particle table into PlumeSoA, step
// on the GPU through the C ABI, unpack.  See gpu_bridge.h.
//
// Compiled against the reference's own headers (datstr/particle.h,
// datstr/thashtab.h, plume/particler.h with the constants of
// plume/parameters.h) by `make -C oracle bridge`; GPU_BRIDGE_SELFTEST adds
// a main() that round-trips a small table through the arrays without a GPU.
#include "gpu_bridge.h"

#include <cstdio>
#include <cstring>

#include "particle.h"
#include "thashtab.h"

PlumeSoA GpuBridge::soa() {
  PlumeSoA s;
  std::memset(&s, 0, sizeof(s));
  s.key = key.data();
  double **d[19] = {&s.x, &s.y, &s.z, &s.vx, &s.vy, &s.vz, &s.vsx, &s.vsy, &s.vsz, &s.mass,
                    &s.h, &s.rho, &s.e, &s.p, &s.Y, &s.gamma, &s.c, &s.T, &s.cp};
  for (int k = 0; k < 19; k++) *d[k] = f[k].data();
  s.phase = phase.data();
  s.bc_type = bc.data();
  s.involved = inv.data();
  return s;
}

size_t GpuBridge::pack(THashTable *P) {
  rows.clear();
  THTIterator it(P);
  for (Particle *p; (p = (Particle *)it.next());) rows.push_back(p);
  const size_t n = rows.size();
  key.resize(n);
  phase.resize(n);
  bc.resize(n);
  inv.resize(n);
  for (auto &v : f) v.assign(n, 0.0);
  for (size_t i = 0; i < n; i++) {
    Particle *p = rows[i];
    key[i] = i;
    for (int a = 0; a < DIMENSION; a++) {
      f[0 + a][i] = p->get_coords()[a];
      f[3 + a][i] = p->get_vel()[a];
      f[6 + a][i] = p->get_smoothed_velocity()[a];
    }
    f[9][i] = p->get_mass();
    f[10][i] = p->get_smlen();
    f[11][i] = p->get_density();
    f[12][i] = p->get_energy();
    f[13][i] = p->get_pressure();
    f[14][i] = p->get_mass_frac();
    f[15][i] = p->get_gamma();
    f[16][i] = p->get_sound_speed();
    f[17][i] = p->get_temperature();
    f[18][i] = p->get_specific_heat_p();
    phase[i] = (uint8_t)p->which_phase();
    bc[i] = (uint8_t)p->get_bc_type();
    inv[i] = (uint8_t)p->get_involved();
  }
  return n;
}

// the values of row r into Particle p
static void put_row(const GpuBridge &b, size_t r, Particle *p) {
  double x[DIMENSION], u[NO_OF_EQNS], vs[DIMENSION];
  u[0] = b.f[11][r];
  u[NO_OF_EQNS - 1] = b.f[12][r];
  for (int a = 0; a < DIMENSION; a++) {
    x[a] = b.f[a][r];
    u[1 + a] = b.f[3 + a][r];
    vs[a] = b.f[6 + a][r];
  }
  p->put_coords(x);
  p->put_state_vars(u);
  p->put_smoothed_velocity(vs);
  p->put_mass(b.f[9][r]);
  p->put_smlen(b.f[10][r]);
  p->put_pressure(b.f[13][r]);
  p->put_mass_frac(b.f[14][r]);
  p->put_gamma(b.f[15][r]);
  p->put_sound_speed(b.f[16][r]);
  p->put_temperature(b.f[17][r]);
  p->put_specific_heat_p(b.f[18][r]);
  p->set_phs_num(b.phase[r]);
  p->put_bc_type(b.bc[r]);
  p->set_involved_flag(b.inv[r]);
}

void GpuBridge::unpack_rows(THashTable *P, size_t n) {
  std::vector<char> alive(rows.size(), 0);
  for (size_t r = 0; r < n; r++) {
    const uint64_t k = key[r];
    if (k < rows.size()) {
      alive[k] = 1;
      put_row(*this, r, rows[k]);
      continue;
    }
    // a row the device created: a new Particle under a key outside the
    // reference's Hilbert keys (first word all ones), state from the row
    unsigned tk[TKEYLENGTH] = {0xffffffffu, (unsigned)(k >> 32), (unsigned)(k & 0xffffffffu)};
    double crd[DIMENSION];
    for (int a = 0; a < DIMENSION; a++) crd[a] = f[a][r];
    Particle *p = new Particle(tk, crd, f[9][r], f[10][r], myid, f[5][r], f[12][r], f[11][r], f[13][r], f[15][r],
                               f[16][r], ng0_P, Cvs_P, Cvg_P, Cva_P, Rg_P, Ra_P);
    put_row(*this, r, p);
    P->add(tk, p);
  }
  for (size_t i = 0; i < rows.size(); i++)  // deleted on the device
    if (!alive[i]) {
      P->remove(rows[i]->getKey());
      delete rows[i];
      rows[i] = nullptr;
    }
}

int GpuBridge::upload() {
  PlumeSoA s = soa();
  return plume_upload(ctx, &s, key.size());
}

int GpuBridge::download(THashTable *P, size_t cap) {
  for (auto &v : f) v.resize(cap);
  key.resize(cap);
  phase.resize(cap);
  bc.resize(cap);
  inv.resize(cap);
  PlumeSoA s = soa();
  size_t n = 0;
  const int rc = plume_download(ctx, &s, cap, &n);
  if (rc) return rc;
  unpack_rows(P, n);
  return PLUME_OK;
}

#ifdef GPU_BRIDGE_SELFTEST
// Round trip without a GPU: a table of 8 particles is packed; the arrays
// are then changed as a device step would change them (rows reordered, one
// deleted, a field updated, one row created) and unpacked; the table must
// show exactly those changes.  The library's version string checks the link.
int main() {
  double mind[DIMENSION] = {-1000., -1000., 0.}, maxd[DIMENSION] = {1000., 1000., 2000.};
  THashTable *P = new THashTable(101, 2017, mind, maxd);
  for (unsigned i = 0; i < 8; i++) {
    unsigned k[TKEYLENGTH] = {i + 1, 7 * i, i};
    double crd[DIMENSION] = {10.0 * i, -5.0 * i, 100.0 + i};
    Particle *p = new Particle(k, crd, 1.0 + i, 50.0, 0, 0., 0., 1., 1., 1.4, 1., ng0_P, Cvs_P, Cvg_P, Cva_P,
                               Rg_P, Ra_P);
    double u[NO_OF_EQNS] = {1.2, 0.1 * i, 0.2 * i, 0.3 * i, 2.0e5 + i};
    p->put_state_vars(u);
    p->put_bc_type(100);
    P->add(k, p);
  }
  GpuBridge b;
  const size_t n = b.pack(P);
  int bad = (n != 8);
  // "device": reverse the rows, drop the last (key 7's row), rho of every
  // row + 1, and one new row with key 8
  GpuBridge d = b;
  for (size_t r = 0; r < 7; r++) {
    const size_t src = 7 - r;
    d.key[r] = b.key[src];
    for (int q = 0; q < 19; q++) d.f[q][r] = b.f[q][src];
    d.phase[r] = b.phase[src];
    d.bc[r] = b.bc[src];
    d.inv[r] = b.inv[src];
    d.f[11][r] += 1.0;
  }
  d.key[7] = 8;
  for (int q = 0; q < 19; q++) d.f[q][7] = b.f[q][0];
  d.f[0][7] = 555.0;
  d.phase[7] = 2;
  d.bc[7] = 0;
  d.inv[7] = 0;
  Particle *gone = b.rows[0];
  const TKey gone_key = gone->getKey();
  std::vector<double> rho_before(8);
  for (size_t i = 0; i < 8; i++) rho_before[i] = b.rows[i]->get_density();
  b.key = d.key;
  for (int q = 0; q < 19; q++) b.f[q] = d.f[q];
  b.phase = d.phase;
  b.bc = d.bc;
  b.inv = d.inv;
  b.unpack_rows(P, 8);
  int count = 0, created = 0;
  THTIterator it(P);
  for (Particle *p; (p = (Particle *)it.next());) {
    count++;
    if (p->getKey().key[0] == 0xffffffffu) {
      created++;
      bad |= (p->get_coords()[0] != 555.0) || (p->get_bc_type() != 0) || (p->which_phase() != 2);
    }
  }
  bad |= (count != 8) || (created != 1) || (P->lookup(gone_key) != nullptr);
  for (size_t i = 1; i < 8; i++) bad |= (b.rows[i]->get_density() != rho_before[i] + 1.0);
  std::printf("gpu_bridge self-test: %s (%d particles, %d created, library %s)\n", bad ? "FAILED" : "ok",
              count, created, plume_version());
  return bad ? 1 : 0;
}
#endif
