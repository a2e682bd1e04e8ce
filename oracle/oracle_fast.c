/*
 * oracle_fast.c -- timing build of the FP32 oracle, for the CPU baseline.
 *
 * TEST INFRASTRUCTURE ONLY (bench.py's CPU-baseline and reference legs); it is
 * not a parity reference.  It compiles the FP32 restatement of
 * axisem_oracle.c with -O3, the host CPU's instruction set and contraction
 * allowed, and adds the stiffness + assembly of the micro-benchmark as a CPU
 * implementation of the reference's algorithm would run it on many cores:
 * elements are coloured so that no two elements of one colour share a global
 * point; per colour, threads take disjoint element ranges, and each element
 * gathers u through igloc_solid, applies the axis mask, the pole's
 * glob_stiffness_*_4 (SOLVER/stiffness_{mono,di,quad}.f90) and the mask of the
 * result, and adds its force into the assembled vector (pdistsum_solid,
 * SOLVER/commun.F90:69-171, with the sums in colour order).
 */
#define REAL float
#define ORC(name) orc_fast_##name
#include "axisem_oracle.c"

#ifdef _OPENMP
#include <omp.h>
#endif

/* Greedy colouring in element order: an element takes the smallest colour no
 * element sharing one of its points has.  order[] receives the elements grouped
 * by colour, colour_start[0..ncol] the groups' bounds; returns ncol (<= 32),
 * or -1 when 32 colours do not suffice. */
int orc_fast_colour_elements(const axg_mesh_desc *d, int32_t *order, int32_t *colour_start) {
  const int64_t ne = d->nel_solid, ng = d->nglob_solid;
  uint32_t *used = (uint32_t *)calloc((size_t)(ng > 0 ? ng : 1), sizeof(uint32_t));
  int32_t *col = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ne > 0 ? ne : 1));
  int ncol = 0;
  for (int64_t e = 0; e < ne; ++e) {
    uint32_t m = 0;
    for (int k = 0; k < 25; ++k) m |= used[d->igloc_solid[25 * e + k] - 1];
    if (m == 0xffffffffu) {
      free(used);
      free(col);
      return -1;
    }
    int c = 0;
    while (m & (1u << c)) ++c;
    col[e] = c;
    if (c + 1 > ncol) ncol = c + 1;
    for (int k = 0; k < 25; ++k) used[d->igloc_solid[25 * e + k] - 1] |= 1u << c;
  }
  int32_t cnt[33] = {0};
  for (int64_t e = 0; e < ne; ++e) cnt[col[e] + 1]++;
  for (int c = 0; c < ncol; ++c) cnt[c + 1] += cnt[c];
  for (int c = 0; c <= ncol; ++c) colour_start[c] = cnt[c];
  for (int64_t e = 0; e < ne; ++e) order[cnt[col[e]]++] = (int32_t)e;
  free(used);
  free(col);
  return ncol;
}

static void mask_el(int pole, int axis, REAL *a1, REAL *a2, REAL *a3) {
  if (!axis) return;
  for (int j = 0; j < 5; ++j) {
    if (pole != AXG_DIPOLE) a1[5 * j] = 0;
    if (pole == AXG_DIPOLE || pole == AXG_QUADPOLE) {
      a2[5 * j] = 0;
      a3[5 * j] = 0;
    }
  }
}

/* f_g = pdistsum_solid(mask(glob_stiffness(mask(u_g)))) on nthreads threads
 * (0: all), gvec layout (nglob, 3); order / colour_start from
 * orc_fast_colour_elements. */
void orc_fast_stiffness_assembled_coloured(const axg_mesh_desc *d, const int32_t *order,
                                           const int32_t *colour_start, int ncol, const REAL *u_g, REAL *f_g,
                                           int nthreads) {
  spec s;
  load_spec(d, &s);
  const int64_t ng = d->nglob_solid;
  const int pole = d->src_type;
  unsigned char *ax = axis_flags(d->nel_solid, d->naxel_solid, d->ax_el_solid);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
#pragma omp parallel num_threads(nthreads)
  {
#pragma omp for schedule(static)
    for (int64_t p = 0; p < 3 * ng; ++p) f_g[p] = 0;
    for (int c = 0; c < ncol; ++c) {
#pragma omp for schedule(static)
      for (int64_t k = colour_start[c]; k < colour_start[c + 1]; ++k) {
        const int64_t e = order[k];
        const int32_t *ig = d->igloc_solid + 25 * e;
        REAL u1[25], u2[25], u3[25], o1[25], o2[25], o3[25];
        for (int q = 0; q < 25; ++q) {
          const int64_t g = ig[q] - 1;
          u1[q] = u_g[g];
          u2[q] = u_g[g + ng];
          u3[q] = u_g[g + 2 * ng];
        }
        mask_el(pole, ax[e], u1, u2, u3);
        if (pole == AXG_MONOPOLE) {
          stiff_mono_el(d, &s, e, ax[e], u1, u3, o1, o3);
          for (int q = 0; q < 25; ++q) o2[q] = 0;
        } else if (pole == AXG_DIPOLE) {
          stiff_di_el(d, &s, e, ax[e], u1, u2, u3, o1, o2, o3);
        } else {
          stiff_quad_el(d, &s, e, ax[e], u1, u2, u3, o1, o2, o3);
        }
        mask_el(pole, ax[e], o1, o2, o3);
        for (int q = 0; q < 25; ++q) {
          const int64_t g = ig[q] - 1;
          f_g[g] += o1[q];
          f_g[g + ng] += o2[q];
          f_g[g + 2 * ng] += o3[q];
        }
      }
    }
  }
  free(ax);
}
