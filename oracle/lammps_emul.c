/*
 * lammps_emul.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * The two pieces of LAMMPS that sit around the reference fix on one MPI
 * rank: creation of periodic ghost images (CommBrick::setup/borders) and
 * the reverse communication that folds ghost forces back into their owners
 * (CommBrick::reverse_comm).  LAMMPS is not vendored by the reference and no
 * version is pinned, so this is a restatement of the published algorithm
 * for a single process with periodic axes; see lbmpsm_oracle.h.
 */
#include <string.h>

#include "lbmpsm_oracle.h"

int orc_make_ghosts(int dimension, const double* boxlo, const double* prd, const int* periodic,
                    double cutghost, int nlocal, int max_images, int* tag, double* x, double* v,
                    double* omega, double* radius, int* owner, int* swap) {
  int nimg = nlocal;
  int iswap = 0;
  for (int i = 0; i < nlocal; ++i) {
    owner[i] = i;
    swap[i] = -1;
  }
  for (int dim = 0; dim < dimension; ++dim) {
    if (!periodic[dim]) continue;
    const double sublo = boxlo[dim], subhi = boxlo[dim] + prd[dim];
    /* both swaps of a dimension scan the atoms present before it */
    const int nlast = nimg;
    for (int ineed = 0; ineed < 2; ++ineed) {
      double lo, hi, shift;
      if (ineed == 0) { /* to the lower neighbour (self): image at +prd */
        lo = -1.0e20;
        hi = sublo + cutghost;
        shift = prd[dim];
      } else { /* to the upper neighbour (self): image at -prd */
        lo = subhi - cutghost;
        hi = 1.0e20;
        shift = -prd[dim];
      }
      for (int i = 0; i < nlast; ++i) {
        if (x[3 * i + dim] >= lo && x[3 * i + dim] <= hi) {
          if (nimg >= max_images) return -1;
          int g = nimg++;
          tag[g] = tag[i];
          for (int c = 0; c < 3; ++c) {
            x[3 * g + c] = x[3 * i + c];
            v[3 * g + c] = v[3 * i + c];
            omega[3 * g + c] = omega[3 * i + c];
          }
          x[3 * g + dim] = x[3 * i + dim] + shift;
          radius[g] = radius[i];
          owner[g] = i;
          swap[g] = iswap;
        }
      }
      ++iswap;
    }
  }
  return nimg;
}

void orc_reverse_comm(int n, int nlocal, const int* owner, const int* swap, int width,
                      double* vals) {
  int maxswap = -1;
  for (int i = nlocal; i < n; ++i)
    if (swap[i] > maxswap) maxswap = swap[i];
  for (int sw = maxswap; sw >= 0; --sw)
    for (int g = nlocal; g < n; ++g)
      if (swap[g] == sw)
        for (int c = 0; c < width; ++c) vals[(long)owner[g] * width + c] += vals[(long)g * width + c];
}
