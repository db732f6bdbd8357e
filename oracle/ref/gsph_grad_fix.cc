// gsph_grad_fix.cc -- project-written calc_gradients that the 1D GSPH
// oracle builds link in place of src/plume/calculate_gradient.cc.
//
// The reference's calc_gradients (calculate_gradient.cc:22-208) clears the
// solution of a particle with 20 or fewer neighbours inside its CUTOFF2*h
// box through `**(ff+i) = 0.` for i < NOEQxDIM (:162-164), while ff is a
// DIMENSION x NO_OF_EQNS array: the writes run past ff on the stack (in 1D
// the ghosts, whose lists are empty, always take that branch), and a
// stack-protected build aborts.  The array is already zero there (:112-120),
// so this version keeps it zero and is otherwise the same computation: the
// sums A_ab = -sum_j dx_a dW_b m_j/rho_j, F_a,q = -sum_j (f_q,i - f_q,j)
// dW_a m_j/rho_j over the list entries inside the box, f = (rho, v, p),
// solved by the reference's own linsolve (sph_lib.cc:161-182) and stored
// with the Particle put_*_d setters.  The 3D builds and the 1D build that
// pins the gradients themselves run the reference's file unchanged, on
// cases where every particle has more than 20 such neighbours.
#include <vector>
#include <cassert>

#include <hashtab.h>
#include <thashtab.h>
#include <particle.h>
#include "particler.h"
#include "constant.h"
#include "sph_header.h"

void calc_gradients(THashTable *P_table)
{
  THTIterator *itr = new THTIterator(P_table);
  Particle *pi = NULL;
  while ((pi = (Particle *)itr->next())) {
    if (pi->is_guest()) continue;
    double xi[DIMENSION], dx[DIMENSION], s[DIMENSION];
    for (int k = 0; k < DIMENSION; k++) xi[k] = *(pi->get_coords() + k);
    const double hi = pi->get_smlen();
    const double supp = CUTOFF2 * hi;
    double AA[DIMENSION][DIMENSION] = {};
    double FF[DIMENSION][NO_OF_EQNS] = {};
    double ff[DIMENSION][NO_OF_EQNS] = {};
    int nreal = 0;
    std::vector<TKey> neighs = pi->get_neighs();
    for (size_t q = 0; q < neighs.size(); q++) {
      Particle *pj = (Particle *)P_table->lookup(neighs[q]);
      assert(pj);
      if (*pi == *pj) continue;
      for (int k = 0; k < DIMENSION; k++) dx[k] = xi[k] - *(pj->get_coords() + k);
      if (!in_support(dx, supp)) continue;
      nreal++;
      const double mj = pj->get_mass(), rhoj = pj->get_density();
      double dwm[DIMENSION];
      for (int k = 0; k < DIMENSION; k++) s[k] = dx[k] / hi;
      for (int k = 0; k < DIMENSION; k++) dwm[k] = d_weight(s, hi, k) * mj / rhoj;
      for (int a = 0; a < DIMENSION; a++)
        for (int b = 0; b < DIMENSION; b++) AA[a][b] -= dx[a] * dwm[b];
      for (int a = 0; a < DIMENSION; a++) {
        FF[a][0] -= (pi->get_density() - pj->get_density()) * dwm[a];
        for (int b = 0; b < DIMENSION; b++)
          FF[a][b + 1] -= (*(pi->get_vel() + b) - *(pj->get_vel() + b)) * dwm[a];
        FF[a][NO_OF_EQNS - 1] -= (pi->get_pressure() - pj->get_pressure()) * dwm[a];
      }
    }
    if (nreal > 20) linsolve(&AA[0][0], &FF[0][0], NO_OF_EQNS, &ff[0][0]);
    double gradU[NOEQxDIM];
    for (int q = 0; q < NO_OF_EQNS; q++)
      for (int a = 0; a < DIMENSION; a++) gradU[q * DIMENSION + a] = ff[a][q];
    pi->put_density_d(gradU);
    pi->put_velocity_u_d(gradU + DIMENSION);
#if CODE_DIMENSION == 3
    pi->put_velocity_v_d(gradU + 2 * DIMENSION);
    pi->put_velocity_w_d(gradU + 3 * DIMENSION);
#endif
    pi->put_pressure_d(gradU + (NO_OF_EQNS - 1) * DIMENSION);
  }
  delete itr;
}
