// driver.cc -- project-written harness that runs the reference solver's own
// hot-path functions (compiled from the Plume-SPH sources by
// oracle/Makefile) on particles read from a binary case file, and dumps the
// particle state after every step plus the neighbour lists of the last step.
//
// TEST INFRASTRUCTURE: it exists to produce golden vectors
// (tests/golden/make_golden.py) that pin the C oracle.  It replaces the
// reference's set-up and I/O (Read_Data, Read_Grid/preprocess, add_air,
// ghosts, inlet) with the particles of the case file, and calls, in the
// order of src/plume/main.cc:217-408 (3D) or :676-729 (1D):
//   timestep, TimeProps::incrtime, search_neighs_consth (3D),
//   adaptive_sml, calc_gradients (USE_GSPH builds), mom_engr_update,
//   smooth_density, smooth_velocity (3D LANS),
//   update_pos, update_particles_in_bucket (3D), TimeProps::ifoutput.
//
// Case file (little endian):
//   char[8] "PLSPHIN1"; int32 dim, nsteps, n, pre_adaptive, step0, dump_last;
//   (nsteps < 0: run until TimeProps::ifend(); dump_last: dump only the last step)
//   double max_time, timeoutput, stat_erupt, end_erupt, sml_phase2;
//   3D only: double mindom[3], del; int32 nb[3]; uint8 flags[nbk];
//            int8 face_index[6*nbk]; double lo[3], hi[3];
//   per particle field arrays (n each): uint64 key; double x,y,z,vx,vy,vz,
//   vsx,vsy,vsz,mass,h,rho,e,p,Y,gamma,c,T,cp; uint8 phase,bc,involved
//   (1D files carry the same 19 double arrays; unused axes are zero).
// Output file:
//   char[8] "PLSPHOU1"; int32 dim, nsteps; then per step:
//   double dt, time; int32 step, ioutput; int64 n; the same field arrays in
//   ascending input-index order (key array = input keys); after the last
//   step: int64 nlists; per need_neigh particle: uint64 key_i, int64 len,
//   uint64 key_j[len] (list order as stored by the reference); GSPH builds
//   (USE_GSPH 1) then append the last step's gradients (dump_gradients).

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>
#include <map>
#include <algorithm>

#include <hashtab.h>
#include <thashtab.h>
#include <bucket.h>
#include <particle.h>
#include <properties.h>
#include "particler.h"
#include "constant.h"
#include "sph_header.h"
#include "plume_gpu.h"
#if CODE_DIMENSION == 3
#include <list>
#include <map>
#include <bnd_image.h>
#endif

static const int NF = 19;

struct Case {
  int dim, nsteps, n, pre_adaptive, step0, dump_last;
  double max_time, timeoutput, stat_erupt, end_erupt, sml_phase2;
  double mindom[3], del;
  int nb[3];
  std::vector<uint8_t> flags;
  std::vector<int8_t> face;
  double lo[3], hi[3];
  std::vector<uint64_t> key;
  std::vector<double> f[NF];
  std::vector<uint8_t> phase, bc, inv;
  // optional wall images (3D): ghost key and image point of each
  std::vector<uint64_t> img_key;
  std::vector<double> img_xyz;
  std::vector<uint8_t> binv;  // per-bucket has_involved (optional)
  int adapt_mode = 0;         // 1: scan_outside_layer + adapt_domain after the loop,
                              // 2: then add_pressure_ghost, 3: add_wall_ghost alone,
                              // 4: add_air alone, 5: setup_erupt alone,
                              // 6: setup_erupt before the loop and
                              //    add_new_erupt in every step
};

static void rd(FILE *fp, void *p, size_t sz, size_t cnt) {
  if (cnt && fread(p, sz, cnt, fp) != cnt) {
    fprintf(stderr, "driver: short read\n");
    exit(2);
  }
}

static void read_case(const char *path, Case &c) {
  FILE *fp = fopen(path, "rb");
  if (!fp) { perror(path); exit(2); }
  char magic[8];
  rd(fp, magic, 1, 8);
  if (memcmp(magic, "PLSPHIN1", 8)) { fprintf(stderr, "bad magic\n"); exit(2); }
  int32_t hdr[6];
  rd(fp, hdr, 4, 6);
  c.dim = hdr[0]; c.nsteps = hdr[1]; c.n = hdr[2]; c.pre_adaptive = hdr[3]; c.step0 = hdr[4];
  c.dump_last = hdr[5];
  double t[5];
  rd(fp, t, 8, 5);
  c.max_time = t[0]; c.timeoutput = t[1]; c.stat_erupt = t[2]; c.end_erupt = t[3];
  c.sml_phase2 = t[4];
  if (c.dim != DIMENSION) { fprintf(stderr, "case dim %d != build %d\n", c.dim, DIMENSION); exit(2); }
  if (c.dim == 3) {
    rd(fp, c.mindom, 8, 3);
    rd(fp, &c.del, 8, 1);
    int32_t nb[3];
    rd(fp, nb, 4, 3);
    for (int a = 0; a < 3; a++) c.nb[a] = nb[a];
    size_t nbk = (size_t)nb[0] * nb[1] * nb[2];
    c.flags.resize(nbk);
    c.face.resize(6 * nbk);
    rd(fp, c.flags.data(), 1, nbk);
    rd(fp, c.face.data(), 1, 6 * nbk);
    rd(fp, c.lo, 8, 3);
    rd(fp, c.hi, 8, 3);
  }
  c.key.resize(c.n);
  rd(fp, c.key.data(), 8, c.n);
  for (int k = 0; k < NF; k++) {
    c.f[k].resize(c.n);
    rd(fp, c.f[k].data(), 8, c.n);
  }
  c.phase.resize(c.n); c.bc.resize(c.n); c.inv.resize(c.n);
  rd(fp, c.phase.data(), 1, c.n);
  rd(fp, c.bc.data(), 1, c.n);
  rd(fp, c.inv.data(), 1, c.n);
  int64_t nimg = 0;
  if (fread(&nimg, 8, 1, fp) == 1 && nimg > 0) {
    c.img_key.resize((size_t)nimg);
    c.img_xyz.resize(3 * (size_t)nimg);
    rd(fp, c.img_key.data(), 8, (size_t)nimg);
    rd(fp, c.img_xyz.data(), 8, 3 * (size_t)nimg);
  }
  int64_t nbinv = 0;
  if (fread(&nbinv, 8, 1, fp) == 1 && nbinv > 0) {
    c.binv.resize((size_t)nbinv);
    rd(fp, c.binv.data(), 1, (size_t)nbinv);
    int32_t mode = 0;
    rd(fp, &mode, 4, 1);
    c.adapt_mode = mode;
  }
  fclose(fp);
}

// particle keys: in 3D key[0] spreads the input index over the 32-bit hash
// range (thashtab.cc:213-222); the 1D table hashes key[0] directly
// (thashtab.cc:205-209), so there key[0] is the index.  key[2] keeps the
// index itself so that every TKey maps back to its input row.
static void pkey(unsigned idx, unsigned k[TKEYLENGTH]) {
  k[0] = (DIMENSION == 1) ? idx : (unsigned)(idx * 2654435761u);
  k[1] = 0;
  k[2] = idx;
}

enum { FX, FY, FZ, FVX, FVY, FVZ, FSX, FSY, FSZ, FM, FH, FRHO, FE, FP, FYF, FG, FC, FT, FCP };

static Particle *make_particle(const Case &c, int i) {
  unsigned k[TKEYLENGTH];
  pkey((unsigned)i, k);
  double crd[DIMENSION];
  for (int a = 0; a < DIMENSION; a++) crd[a] = c.f[FX + a][i];
#if CODE_DIMENSION == 1
  Particle *p = new Particle(k, crd, c.f[FM][i], c.f[FH][i], c.f[FRHO][i], c.f[FVX][i],
                             c.f[FP][i], c.f[FG][i], c.f[FC][i], c.bc[i], c.inv[i]);
#else
  Particle *p = new Particle(k, crd, c.f[FM][i], c.f[FH][i], 0, 0., 0., 1., 1., 1.4, 1.,
                             ng0_P, Cvs_P, Cvg_P, Cva_P, Rg_P, Ra_P);
#endif
  double u[NO_OF_EQNS];
  u[0] = c.f[FRHO][i];
  for (int a = 0; a < DIMENSION; a++) u[1 + a] = c.f[FVX + a][i];
  u[NO_OF_EQNS - 1] = c.f[FE][i];
  p->put_state_vars(u);
  p->put_coords(crd);
  p->put_mass(c.f[FM][i]);
  p->put_smlen(c.f[FH][i]);
  p->put_pressure(c.f[FP][i]);
  p->put_mass_frac(c.f[FYF][i]);
  p->put_gamma(c.f[FG][i]);
  p->put_sound_speed(c.f[FC][i]);
  p->put_temperature(c.f[FT][i]);
  p->put_specific_heat_p(c.f[FCP][i]);
  double vs[DIMENSION];
  for (int a = 0; a < DIMENSION; a++) vs[a] = c.f[FSX + a][i];
  p->put_smoothed_velocity(vs);
  p->set_phs_num(c.phase[i]);
  p->put_bc_type(c.bc[i]);
  p->set_involved_flag(c.inv[i]);
  p->put_guest_flag(false);
  return p;
}

// a particle of the case (key pkey(row)) rather than one the reference
// created during the run
static bool case_particle(Particle *p, const Case &c) {
  const unsigned r = p->getKey().key[2];
  if (r >= (unsigned)c.n) return false;
  unsigned k[TKEYLENGTH];
  pkey(r, k);
  for (int q = 0; q < TKEYLENGTH; q++)
    if (p->getKey().key[q] != k[q]) return false;
  return true;
}

static void dump_state(FILE *fo, THashTable *P, const Case &c, const TimeProps &tp, double dt) {
  std::vector<std::pair<unsigned, Particle *>> rows;
  THTIterator it(P);
  Particle *p;
  while ((p = (Particle *)it.next()))
    if (case_particle(p, c)) rows.push_back(std::make_pair(p->getKey().key[2], p));
  std::sort(rows.begin(), rows.end(),
            [](const std::pair<unsigned, Particle *> &a, const std::pair<unsigned, Particle *> &b) {
              return a.first < b.first;
            });
  double hd[2] = { dt, tp.time };
  int32_t hi[2] = { tp.step, tp.ioutput };
  int64_t n = (int64_t)rows.size();
  fwrite(hd, 8, 2, fo);
  fwrite(hi, 4, 2, fo);
  fwrite(&n, 8, 1, fo);
  std::vector<uint64_t> kk(n);
  for (int64_t r = 0; r < n; r++) kk[r] = c.key[rows[r].first];
  fwrite(kk.data(), 8, n, fo);
  std::vector<double> col(n);
  for (int f = 0; f < NF; f++) {
    for (int64_t r = 0; r < n; r++) {
      Particle *q = rows[r].second;
      double v = 0;
      switch (f) {
      case FX: case FY: case FZ:
        v = (f - FX < DIMENSION) ? q->get_coords()[f - FX] : 0.; break;
      case FVX: case FVY: case FVZ:
        v = (f - FVX < DIMENSION) ? q->get_vel()[f - FVX] : 0.; break;
      case FSX: case FSY: case FSZ:
        v = (f - FSX < DIMENSION) ? q->get_smoothed_velocity()[f - FSX] : 0.; break;
      case FM: v = q->get_mass(); break;
      case FH: v = q->get_smlen(); break;
      case FRHO: v = q->get_density(); break;
      case FE: v = q->get_energy(); break;
      case FP: v = q->get_pressure(); break;
      case FYF: v = q->get_mass_frac(); break;
      case FG: v = q->get_gamma(); break;
      case FC: v = q->get_sound_speed(); break;
      case FT: v = q->get_temperature(); break;
      case FCP: v = q->get_specific_heat_p(); break;
      }
      col[r] = v;
    }
    fwrite(col.data(), 8, n, fo);
  }
  std::vector<uint8_t> b(n);
  for (int64_t r = 0; r < n; r++) b[r] = (uint8_t)rows[r].second->which_phase();
  fwrite(b.data(), 1, n, fo);
  for (int64_t r = 0; r < n; r++) b[r] = (uint8_t)rows[r].second->get_bc_type();
  fwrite(b.data(), 1, n, fo);
  for (int64_t r = 0; r < n; r++) b[r] = (uint8_t)rows[r].second->get_involved();
  fwrite(b.data(), 1, n, fo);
}

static void dump_lists(FILE *fo, THashTable *P, const Case &c) {
  std::vector<std::pair<unsigned, Particle *>> rows;
  THTIterator it(P);
  Particle *p;
  while ((p = (Particle *)it.next()))
    if (p->need_neigh()) rows.push_back(std::make_pair(p->getKey().key[2], p));
  std::sort(rows.begin(), rows.end(),
            [](const std::pair<unsigned, Particle *> &a, const std::pair<unsigned, Particle *> &b) {
              return a.first < b.first;
            });
  int64_t nl = (int64_t)rows.size();
  fwrite(&nl, 8, 1, fo);
  for (auto &r : rows) {
    std::vector<TKey> nb = r.second->get_neighs();
    uint64_t ki = c.key[r.first];
    int64_t len = (int64_t)nb.size();
    fwrite(&ki, 8, 1, fo);
    fwrite(&len, 8, 1, fo);
    std::vector<uint64_t> kj(len);
    for (int64_t q = 0; q < len; q++) kj[q] = c.key[nb[q].key[2]];
    fwrite(kj.data(), 8, len, fo);
  }
}

#if USE_GSPH != 0
// GSPH builds: the gradients that calc_gradients stored in the last step,
// char[4] "GRAD"; int64 n; uint64 key[n]; then per particle (D+2)*D doubles
// (d rho, d v_0 .. d v_D-1, d p; x_k fastest), input-index order.
static void dump_gradients(FILE *fo, THashTable *P, const Case &c) {
  std::vector<std::pair<unsigned, Particle *>> rows;
  THTIterator it(P);
  Particle *p;
  while ((p = (Particle *)it.next())) rows.push_back(std::make_pair(p->getKey().key[2], p));
  std::sort(rows.begin(), rows.end(),
            [](const std::pair<unsigned, Particle *> &a, const std::pair<unsigned, Particle *> &b) {
              return a.first < b.first;
            });
  fwrite("GRAD", 1, 4, fo);
  int64_t n = (int64_t)rows.size();
  fwrite(&n, 8, 1, fo);
  for (auto &r : rows) {
    uint64_t k = c.key[r.first];
    fwrite(&k, 8, 1, fo);
  }
  for (auto &r : rows) {
    Particle *q = r.second;
    const double *g[5] = { q->get_density_derivative(), q->get_velocity_u_derivative(),
                           q->get_velocity_v_derivative(), q->get_velocity_w_derivative(),
                           q->get_pressure_derivative() };
    const int idx3[5] = { 0, 1, 2, 3, 4 }, idx1[3] = { 0, 1, 4 };
    const int nq = DIMENSION + 2;
    for (int a = 0; a < nq; a++) fwrite(g[DIMENSION == 3 ? idx3[a] : idx1[a]], 8, DIMENSION, fo);
  }
}
#endif

int main(int argc, char **argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s case.bin out.bin\n", argv[0]);
    return 2;
  }
  Case c;
  read_case(argv[1], c);

  MatProps *matprops = new MatProps();
  matprops->smoothing_length = c.sml_phase2;
  TimeProps *tp = new TimeProps();
  tp->time = 0.;  // never initialised by the reference (properties.h:48-58)
  tp->max_time = tp->ndmax_time = c.max_time;
  tp->timeoutput = c.timeoutput;
  tp->ndtimeoutput = c.timeoutput;
  tp->TIME_SCALE = 1.;
  tp->stat_erupt = c.stat_erupt;
  tp->end_erupt = c.end_erupt;
  tp->step = c.step0;
  tp->ioutput = 0;
  tp->max_steps = 1 << 30;
  SimProps *simprops = new SimProps();

  double mind[DIMENSION], maxd[DIMENSION];
  for (int a = 0; a < DIMENSION; a++) {
    mind[a] = (c.dim == 3) ? c.mindom[a] : -1.0;
    maxd[a] = (c.dim == 3) ? c.mindom[a] + c.nb[a] * c.del : 1.0;
  }
  int psize = (c.dim == 1) ? c.n + 16 : 200003;
  THashTable *P = new THashTable(psize, 2017, mind, maxd);
  for (int i = 0; i < c.n; i++) {
    unsigned k[TKEYLENGTH];
    pkey((unsigned)i, k);
    P->add(k, make_particle(c, i));
  }

#if CODE_DIMENSION == 1
  {
    // every particle is a neighbour of every need_neigh particle,
    // in creation order (add_air.cc:470-479)
    std::vector<TKey> all;
    for (int i = 0; i < c.n; i++) {
      unsigned k[TKEYLENGTH];
      pkey((unsigned)i, k);
      all.push_back(TKey(k));
    }
    THTIterator it(P);
    Particle *p;
    while ((p = (Particle *)it.next()))
      if (p->need_neigh()) p->put_neighs(all);
  }
  HashTable *BG = NULL;
#else
  HashTable *BG = new HashTable(20011, 2017, mind, maxd);
  int nbx = c.nb[0], nby = c.nb[1], nbz = c.nb[2];
  auto bkey = [&](int i, int j, int k, unsigned out[KEYLENGTH]) {
    unsigned idx = (unsigned)((k * nby + j) * nbx + i);
    out[0] = (unsigned)((idx + 1) * 2654435761u);
    out[1] = idx;
  };
  std::vector<Bucket *> bucks((size_t)nbx * nby * nbz);
  bool explicit_types = false;
  for (size_t b = 0; b < bucks.size(); b++)
    explicit_types |= (c.flags[b] & (PLUME_BUCKET_UNDERGROUND | PLUME_BUCKET_PRESS_BC)) != 0;
  for (int i = 0; i < nbx; i++)
    for (int j = 0; j < nby; j++)
      for (int k = 0; k < nbz; k++) {
        size_t b = ((size_t)k * nby + j) * nbx + i;
        unsigned key[KEYLENGTH];
        bkey(i, j, k, key);
        double minx[3] = { c.mindom[0] + i * c.del, c.mindom[1] + j * c.del, c.mindom[2] + k * c.del };
        double maxx[3] = { c.mindom[0] + (i + 1) * c.del, c.mindom[1] + (j + 1) * c.del,
                           c.mindom[2] + (k + 1) * c.del };
        Key neigh[NEIGH_SIZE];
        int nproc[NEIGH_SIZE];
        int q = 0;
        // neighbour order of preprocess.cc:287-313
        for (int ii = i - 1; ii < i + 2; ii++)
          for (int jj = j - 1; jj < j + 2; jj++)
            for (int kk = k - 1; kk < k + 2; kk++) {
              if (ii > -1 && ii < nbx && jj > -1 && jj < nby && kk > -1 && kk < nbz) {
                unsigned nk[KEYLENGTH];
                bkey(ii, jj, kk, nk);
                neigh[q] = Key(nk);
                nproc[q] = (ii == i && jj == j && kk == k) ? -2 : 0;
              } else {
                unsigned zk[KEYLENGTH] = { 0, 0 };
                neigh[q] = Key(zk);
                nproc[q] = -1;
              }
              q++;
            }
        uint8_t fl = c.flags[b];
        int bt[6];
        for (int a = 0; a < 6; a++) bt[a] = c.face[6 * b + a];
        // bucket types of determine_bucket_type (preprocess.cc:404-439)
        // (explicit UNDERGROUND / PRESS_BC flags, else an absorbing bucket
        // is read as below or beside the ground)
        int btype = OVERGROUND;
        if (fl & PLUME_BUCKET_MIXED)
          btype = MIXED;
        else if (fl & PLUME_BUCKET_UNDERGROUND)
          btype = UNDERGROUND;
        else if (fl & PLUME_BUCKET_PRESS_BC)
          btype = PRESS_BC;
        else if ((fl & PLUME_BUCKET_ABSORBING) && !explicit_types)
          btype = (bt[4] == -1 && bt[5] == -1) ? UNDERGROUND : PRESS_BC;
        double flat[6] = { c.lo[0], c.hi[0], c.lo[1], c.hi[1], c.lo[2], c.hi[2] };
        double elev[4] = { c.lo[2], c.lo[2], c.lo[2], c.lo[2] };
        Bucket *bk = new Bucket(key, minx, maxx, btype, elev, 0, nproc, neigh, bt, flat);
        if (!(fl & PLUME_BUCKET_INACTIVE)) bk->mark_active();
        if (!c.binv.empty()) {
          bk->set_has_no_involved();
          if (c.binv[b] & 1) bk->set_has_potential_involved(true);
          if (c.binv[b] & 2) bk->set_has_involved(true);
        } else if (fl & PLUME_BUCKET_ABSORBING) {
          bk->set_has_no_involved();
        } else {
          bk->set_has_involved(true);
        }
        bucks[b] = bk;
        BG->add(key, bk);
      }
  // particles into buckets by position, in input order
  std::vector<std::vector<TKey>> plists(bucks.size());
  for (int i = 0; i < c.n; i++) {
    int b3[3];
    for (int a = 0; a < 3; a++) {
      double x = c.f[FX + a][i];
      int b = (int)((x - c.mindom[a]) / c.del);
      if (b < 0) b = 0;
      if (b > c.nb[a] - 1) b = c.nb[a] - 1;
      while (b > 0 && x < c.mindom[a] + b * c.del) b--;
      while (b < c.nb[a] - 1 && x >= c.mindom[a] + (b + 1) * c.del) b++;
      b3[a] = b;
    }
    size_t b = ((size_t)b3[2] * nby + b3[1]) * nbx + b3[0];
    unsigned k[TKEYLENGTH];
    pkey((unsigned)i, k);
    plists[b].push_back(TKey(k));
    Bucket *bk = bucks[b];
    switch (c.bc[i]) {
    case 100: case 99: bk->set_real_particles(true); break;
    case 2: bk->set_wall_ghost_particles(true); break;
    case 1: bk->set_pressure_ghost_particles(true); break;
    case 0: bk->set_erupt_ghost_particles(true); break;
    }
  }
  for (size_t b = 0; b < bucks.size(); b++) bucks[b]->put_plist(plists[b]);
#if defined(PLUME_ADJUST_DOMAIN)
  // mode 6: the initial vent duct of setup_erupt (main.cc:156) before the
  // loop, and the per-step inlet add_new_erupt in it (main.cc:414-421)
  if (c.adapt_mode == 6) setup_erupt(0, P, BG, tp, matprops, simprops, 1);
#endif
  // wall images (the table search_bnd_images builds, bnd_image.cc:35-245):
  // the ghost's key and the image point come from the case, the bucket
  // is the one containing the image
  std::list<BndImage> Image_table;
  {
    std::map<uint64_t, int> row;
    for (int i = 0; i < c.n; i++) row[c.key[i]] = i;
    for (size_t q = 0; q < c.img_key.size(); q++) {
      auto it = row.find(c.img_key[q]);
      if (it == row.end()) continue;
      double refc[3] = { c.img_xyz[3 * q], c.img_xyz[3 * q + 1], c.img_xyz[3 * q + 2] };
      int b3[3];
      for (int a = 0; a < 3; a++) {
        int b = (int)floor((refc[a] - c.mindom[a]) / c.del);
        if (b < 0) b = 0;
        if (b > c.nb[a] - 1) b = c.nb[a] - 1;
        while (b > 0 && refc[a] < c.mindom[a] + b * c.del) b--;
        while (b < c.nb[a] - 1 && refc[a] >= c.mindom[a] + (b + 1) * c.del) b++;
        b3[a] = b;
      }
      unsigned bk2[KEYLENGTH], gk[TKEYLENGTH];
      bkey(b3[0], b3[1], b3[2], bk2);
      pkey((unsigned)it->second, gk);
      Image_table.push_back(BndImage(0, 0, bk2, gk, refc));
    }
  }
  // boundary condition before the loop (main.cc:196)
  if (!Image_table.empty()) apply_bcond(0, P, BG, matprops, Image_table);
#endif

  FILE *fo = fopen(argv[2], "wb");
  if (!fo) { perror(argv[2]); return 2; }
  fwrite("PLSPHOU1", 1, 8, fo);
  // the step count is patched in after the run when nsteps < 0 or dump_last
  int32_t hdr[2] = { c.dim, 0 };
  fwrite(hdr, 4, 2, fo);

#if CODE_DIMENSION == 1
  if (c.pre_adaptive) adaptive_sml(0, P);  // main.cc:643-649
#endif
  int lost = 0;
  int ndumped = 0;
  // ORACLE_STEP_TIMES set: the wall time of every step on stderr (the
  // reference's single-thread speed, beside the oracle port's)
  const bool step_times = getenv("ORACLE_STEP_TIMES") != NULL;
  for (int st = 0; c.nsteps < 0 ? !tp->ifend() : st < c.nsteps; st++) {
    const auto t_step = std::chrono::steady_clock::now();
#if CODE_DIMENSION == 1
    double dt = timestep(P, tp);
    tp->incrtime(&dt);
    adaptive_sml(0, P);
#if USE_GSPH != 0
    calc_gradients(P);  // main.cc:697-699
#endif
    mom_engr_update(0, P, tp, simprops);
    smooth_density(P);
    update_pos(P, tp, matprops);
#else
    double dt = timestep(BG, P, tp);
    tp->incrtime(&dt);
    search_neighs_consth(0, P, BG);
    if ((tp->step) % SML_UPDATE_INT == 0) adaptive_sml(0, P);
#if USE_GSPH != 0
    calc_gradients(P);  // main.cc:341-343
#endif
    mom_engr_update(0, P, tp, simprops);
    smooth_density(P);
#if HAVE_TURBULENCE_LANS != 0
    smooth_velocity(P);
#endif
    update_pos(P, tp, matprops);
    update_particles_in_bucket(0, P, BG, &lost);
#if defined(PLUME_ADJUST_DOMAIN)
    if (c.adapt_mode == 6 && tp->iferupt()) add_new_erupt(0, P, BG, tp, matprops, simprops, dt);  // main.cc:414-421
#endif
    if (!Image_table.empty()) apply_bcond(0, P, BG, matprops, Image_table);  // main.cc:468
#endif
    if (step_times)
      fprintf(stderr, "STEP_SECONDS %d %.6f\n", tp->step,
              std::chrono::duration<double>(std::chrono::steady_clock::now() - t_step).count());
    tp->ifoutput();
    bool last = (c.nsteps < 0) ? tp->ifend() : (st == c.nsteps - 1);
    if (!c.dump_last || last) {
      dump_state(fo, P, c, *tp, dt);
      ndumped++;
    }
  }
#if CODE_DIMENSION == 1 && defined(PLUME_WRITE_CSV)
  // the shock-tube text output of the final state (main.cc:749): appends
  // to pvplot_out.csv in the working directory.  The table iterates in
  // ascending key order here (every key hashes to slot 0), which is the
  // case's row order.
  write_csv(0, 1, P, tp);
#endif
#if CODE_DIMENSION == 3 && defined(PLUME_ADJUST_DOMAIN)
  // domain growth after the last step (main.cc:433-436, 257-265): the scan,
  // then adapt_domain when it asks for it; the particles after it are an
  // extra dumped record
  int adapt_n = 0;
  if (c.adapt_mode == 5) {
    // the initial vent duct of setup_erupt (setup_erupt.cc:44-388,
    // main.cc:156): new erupt ghosts, displaced particles removed
    setup_erupt(0, P, BG, tp, matprops, simprops, 1);
    dump_state(fo, P, c, *tp, 0.0);
    ndumped++;
  } else if (c.adapt_mode == 3 || c.adapt_mode == 4) {
    // the wall-ghost layers of add_wall_ghost alone (main.cc:279), or the
    // air of add_air in the empty buckets (add_air.cc:490-795)
    if (c.adapt_mode == 3)
      add_wall_ghost(P, BG, simprops, matprops, tp, 1, 0);
    else
      add_air(P, BG, matprops, simprops, 1, 0);
    dump_state(fo, P, c, *tp, 0.0);
    ndumped++;
  } else if (c.adapt_mode == 6) {
    // the duct and the injected particles are the born record below
  } else if (c.adapt_mode) {
    adapt_n = scan_outside_layer(P, BG, 1, 0);
    if (adapt_n) adapt_domain(P, BG, matprops, 1, 0);
    // the pressure-ghost layers that follow an adaptation (main.cc:265-271)
    if (adapt_n && c.adapt_mode == 2) add_pressure_ghost(P, BG, simprops, matprops, tp, 1, 0);
    dump_state(fo, P, c, *tp, 0.0);
    ndumped++;
  }
#endif
  dump_lists(fo, P, c);
#if USE_GSPH != 0
  dump_gradients(fo, P, c);
#endif
#if CODE_DIMENSION == 3 && defined(PLUME_ADJUST_DOMAIN)
  // char[4] "ADPT"; int32 adapt; int64 nbk; uint8 has_involved per bucket
  if (c.adapt_mode) {
    fwrite("ADPT", 1, 4, fo);
    int32_t a = adapt_n;
    fwrite(&a, 4, 1, fo);
    int64_t nbk = (int64_t)bucks.size();
    fwrite(&nbk, 8, 1, fo);
    for (size_t b = 0; b < bucks.size(); b++) {
      uint8_t st = (uint8_t)bucks[b]->get_has_involved();
      fwrite(&st, 1, 1, fo);
    }
    // char[4] "PGHO"; int64 n; the particles created during the run (by
    // add_pressure_ghost), ordered by key: double x, y, z, vx, vy, vz, vsx,
    // vsy, vsz, m, h, rho, e, p, Y, gamma, c, T, cp (n each), then uint8
    // phase, bc_type, involved; then uint8 active per bucket
    std::vector<Particle *> born;
    THTIterator it(P);
    Particle *p;
    while ((p = (Particle *)it.next()))
      if (!case_particle(p, c)) born.push_back(p);
    std::sort(born.begin(), born.end(), [](Particle *a, Particle *b) { return a->getKey() < b->getKey(); });
    fwrite("PGHO", 1, 4, fo);
    int64_t nn = (int64_t)born.size();
    fwrite(&nn, 8, 1, fo);
    std::vector<double> col(born.size());
    for (int f = 0; f < NF; f++) {
      for (size_t r = 0; r < born.size(); r++) {
        Particle *q = born[r];
        double v = 0;
        switch (f) {
        case FX: case FY: case FZ: v = q->get_coords()[f - FX]; break;
        case FVX: case FVY: case FVZ: v = q->get_vel()[f - FVX]; break;
        case FSX: case FSY: case FSZ: v = q->get_smoothed_velocity()[f - FSX]; break;
        case FM: v = q->get_mass(); break;
        case FH: v = q->get_smlen(); break;
        case FRHO: v = q->get_density(); break;
        case FE: v = q->get_energy(); break;
        case FP: v = q->get_pressure(); break;
        case FYF: v = q->get_mass_frac(); break;
        case FG: v = q->get_gamma(); break;
        case FC: v = q->get_sound_speed(); break;
        case FT: v = q->get_temperature(); break;
        case FCP: v = q->get_specific_heat_p(); break;
        }
        col[r] = v;
      }
      fwrite(col.data(), 8, born.size(), fo);
    }
    std::vector<uint8_t> bb(born.size());
    for (size_t r = 0; r < born.size(); r++) bb[r] = (uint8_t)born[r]->which_phase();
    fwrite(bb.data(), 1, born.size(), fo);
    for (size_t r = 0; r < born.size(); r++) bb[r] = (uint8_t)born[r]->get_bc_type();
    fwrite(bb.data(), 1, born.size(), fo);
    for (size_t r = 0; r < born.size(); r++) bb[r] = (uint8_t)born[r]->get_involved();
    fwrite(bb.data(), 1, born.size(), fo);
    for (size_t b = 0; b < bucks.size(); b++) {
      uint8_t act = (uint8_t)bucks[b]->is_active();
      fwrite(&act, 1, 1, fo);
    }
  }
#endif
  fseek(fo, 12, SEEK_SET);
  int32_t nd = ndumped;
  fwrite(&nd, 4, 1, fo);
  fclose(fo);
  (void)lost;
  (void)BG;
  return 0;
}
