/*
 * axisem_oracle.c -- CPU restatement of the AxiSEM SOLVER time loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA path is checked
 * against; nothing in the product links or calls it.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm use it.
 *
 * It restates, in the reference's element-local layouts and in the same
 * arithmetic order, the Fortran routines on the hot path:
 *   mxm_4 / vxm_4 / outerprod_4 / mxm_cg4_sparse_{a,b,c}   SOLVER/unrolled_loops.f90:76-229
 *   glob_stiffness_mono_4                                   SOLVER/stiffness_mono.f90:60-157
 *   glob_stiffness_di_4                                     SOLVER/stiffness_di.f90:60-256
 *   glob_stiffness_quad_4                                   SOLVER/stiffness_quad.f90:238-414
 *   glob_fluid_stiffness_4                                  SOLVER/stiffness_fluid.f90:139-216
 *   glob_anel_stiffness_{mono,di,quad}_cg4                  SOLVER/stiffness_mono.f90:511,
 *                                                           stiffness_di.f90:727, stiffness_quad.f90:672
 *   time_step_memvars_cg4, compute_strain_att_el_cg4        SOLVER/attenuation.f90:81-202,471-535
 *   fast_correct                                            SOLVER/attenuation.f90:1139-1155
 *   axisym_gradient_solid_el_cg4, f_over_s_solid_el_cg4     SOLVER/pointwise_derivatives.f90:55-75,216-250
 *   apply_axis_mask_*                                       SOLVER/apply_masks.f90:40-98
 *   pdistsum_solid / pdistsum_fluid (serial)                SOLVER/commun.F90:69-171,180-283
 *   bdry_copy2fluid / bdry_copy2solid                       SOLVER/time_evol_wave.F90:1532-1611
 *   add_source_el / add_source_fl                           SOLVER/time_evol_wave.F90:1062-1097
 *   runtime_info blow-up check                              SOLVER/time_evol_wave.F90:1042-1054
 *   nc_compute_recfile_seis_bare                            SOLVER/seismograms.f90:783-820
 *   sf_time_loop_newmark                                    SOLVER/time_evol_wave.F90:264-502
 *   symplectic_time_loop                                    SOLVER/time_evol_wave.F90:516-742
 *   axisym_gradient_solid / _fluid, f_over_s_solid / _fluid,
 *   dsdf_solid_allaxis / dsdf_fluid_allaxis                 SOLVER/pointwise_derivatives.f90:130-178,329-545
 *   compute_strain                                          SOLVER/time_evol_wave.F90:1264-1410
 *   dump_disp_global, dump_velo_global, dump_disp,
 *   dump_velo_dchi                                          SOLVER/wavefields_io.f90:840-1115
 *
 * Compiled twice: REAL=float (the reference's realkind=sp build) and
 * REAL=double (realkind=dp, the FP64 oracle).  Mixed-precision expressions
 * of the reference (FP64 constants deltat, half_dt, third, two; FP64 SLS
 * coefficients) are evaluated in double and rounded to REAL, as Fortran does.
 * Build with -ffp-contract=off so that no FMA changes the rounding.  With
 * -fopenmp the element (and point) loops run on threads; every element's
 * arithmetic is unchanged and the assembly stays serial in the reference's
 * order, so the results do not depend on the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "axisem_gb300.h"

#ifndef REAL
#define REAL float
#endif
#ifndef ORC
#define ORC(name) orc_f32_##name
#endif

typedef REAL mat5[25]; /* (0:4,0:4) column-major: a(i,j) = a[i + 5*j] */
typedef REAL vec5[5];

#define A(a, i, j) ((a)[(i) + 5 * (j)])

/* ---------------------------------------------------------------- helpers */

static void load_mat(mat5 dst, const float *src) {
  for (int k = 0; k < 25; ++k) dst[k] = (REAL)src[k];
}

/* mxm_4: c(i,j) = sum(a(i,:) * b(:,j)), summed k = 0..4 */
static void mxm_4(const REAL *a, const REAL *b, REAL *c) {
  for (int j = 0; j < 5; ++j)
    for (int i = 0; i < 5; ++i) {
      REAL s = A(a, i, 0) * A(b, 0, j);
      s = s + A(a, i, 1) * A(b, 1, j);
      s = s + A(a, i, 2) * A(b, 2, j);
      s = s + A(a, i, 3) * A(b, 3, j);
      s = s + A(a, i, 4) * A(b, 4, j);
      A(c, i, j) = s;
    }
}

/* vxm_4: c(j) = sum(a * b(:,j)) */
static void vxm_4(const REAL *a, const REAL *b, REAL *c) {
  for (int j = 0; j < 5; ++j) {
    REAL s = a[0] * A(b, 0, j);
    s = s + a[1] * A(b, 1, j);
    s = s + a[2] * A(b, 2, j);
    s = s + a[3] * A(b, 3, j);
    s = s + a[4] * A(b, 4, j);
    c[j] = s;
  }
}

/* outerprod_4: o(i,j) = a(i) * b(j) */
static void outerprod_4(const REAL *a, const REAL *b, REAL *o) {
  for (int j = 0; j < 5; ++j)
    for (int i = 0; i < 5; ++i) A(o, i, j) = a[i] * b[j];
}

/* mxm_cg4_sparse_a: a(1:4) sparse left factor at (1,1),(1,3),(3,1),(3,3) */
static void mxm_cg4_sparse_a(const REAL *a, const REAL *b, REAL *c) {
  for (int k = 0; k < 25; ++k) c[k] = 0;
  for (int j = 0; j < 5; ++j) {
    A(c, 1, j) = a[0] * A(b, 1, j) + a[1] * A(b, 3, j);
    A(c, 3, j) = a[2] * A(b, 1, j) + a[3] * A(b, 3, j);
  }
}

/* mxm_cg4_sparse_b: b(1:4) sparse right factor */
static void mxm_cg4_sparse_b(const REAL *a, const REAL *b, REAL *c) {
  for (int k = 0; k < 25; ++k) c[k] = 0;
  for (int i = 0; i < 5; ++i) {
    A(c, i, 1) = A(a, i, 1) * b[0] + A(a, i, 3) * b[2];
    A(c, i, 3) = A(a, i, 1) * b[1] + A(a, i, 3) * b[3];
  }
}

/* mxm_cg4_sparse_c: (a b) at the four cg4 points only */
static void mxm_cg4_sparse_c(const REAL *a, const REAL *b, REAL *c) {
  const int ii[4] = {1, 1, 3, 3}, jj[4] = {1, 3, 1, 3};
  for (int p = 0; p < 4; ++p) {
    REAL s = A(a, ii[p], 0) * A(b, 0, jj[p]);
    s = s + A(a, ii[p], 1) * A(b, 1, jj[p]);
    s = s + A(a, ii[p], 2) * A(b, 2, jj[p]);
    s = s + A(a, ii[p], 3) * A(b, 3, jj[p]);
    s = s + A(a, ii[p], 4) * A(b, 4, jj[p]);
    c[p] = s;
  }
}

typedef struct spec {
  mat5 G1, G1T, G2, G2T;
  vec5 G0;
} spec;

static void load_spec(const axg_mesh_desc *d, spec *s) {
  load_mat(s->G1, d->G1);
  load_mat(s->G1T, d->G1T);
  load_mat(s->G2, d->G2);
  load_mat(s->G2T, d->G2T);
  for (int k = 0; k < 5; ++k) s->G0[k] = (REAL)d->G0[k];
}

static unsigned char *axis_flags(int nel, int nax, const int32_t *ax_el) {
  unsigned char *f = (unsigned char *)calloc((size_t)(nel > 0 ? nel : 1), 1);
  for (int k = 0; k < nax; ++k) f[ax_el[k] - 1] = 1;
  return f;
}

#define MS(t) (d->m_solid[t] + off)
#define M0(t) (d->m0_solid[t] + off0)

/* ------------------------------------------------- solid stiffness (per element) */

/* glob_stiffness_mono_4, SOLVER/stiffness_mono.f90:60-157 */
static void stiff_mono_el(const axg_mesh_desc *d, const spec *s, int64_t e, int axis,
                          const REAL *us_, const REAL *uz_, REAL *out_s, REAL *out_z) {
  const int64_t off = 25 * e, off0 = 5 * e;
  mat5 us, uz, X1, X2, X3, X4, S1s, S2s, S1z, S2z, ls, lz;
  mat5 m1, m2, m3, m4, mw1, m11s, m21s, m41s, m12s, m22s, m32s, m42s, m11z, m21z, m41z;
  memcpy(us, us_, sizeof us);
  memcpy(uz, uz_, sizeof uz);
  load_mat(m1, MS(AXG_M_1)); load_mat(m2, MS(AXG_M_2));
  load_mat(m3, MS(AXG_M_3)); load_mat(m4, MS(AXG_M_4));
  load_mat(mw1, MS(AXG_M_W1));
  load_mat(m11s, MS(AXG_M11S)); load_mat(m21s, MS(AXG_M21S)); load_mat(m41s, MS(AXG_M41S));
  load_mat(m12s, MS(AXG_M12S)); load_mat(m22s, MS(AXG_M22S)); load_mat(m32s, MS(AXG_M32S));
  load_mat(m42s, MS(AXG_M42S));
  load_mat(m11z, MS(AXG_M11Z)); load_mat(m21z, MS(AXG_M21Z)); load_mat(m41z, MS(AXG_M41Z));

  const REAL *GT = axis ? s->G1T : s->G2T;
  const REAL *G = axis ? s->G1 : s->G2;
  mxm_4(GT, us, X1);
  mxm_4(GT, uz, X2);
  mxm_4(us, s->G2, X3);
  mxm_4(uz, s->G2, X4);

  for (int k = 0; k < 25; ++k) {
    ls[k] = m4[k] * X4[k] + m2[k] * X3[k] + m1[k] * X1[k] + m3[k] * X2[k] + us[k] * mw1[k];
    S1s[k] = m11s[k] * X3[k] + m21s[k] * X1[k] + m12s[k] * X4[k] + m22s[k] * X2[k] + m1[k] * us[k];
    S2s[k] = m11s[k] * X1[k] + m41s[k] * X3[k] + m32s[k] * X2[k] + m42s[k] * X4[k] + m2[k] * us[k];
    S1z[k] = m11z[k] * X4[k] + m21z[k] * X2[k] + m32s[k] * X3[k] + m22s[k] * X1[k] + m3[k] * us[k];
    S2z[k] = m11z[k] * X2[k] + m41z[k] * X4[k] + m12s[k] * X1[k] + m42s[k] * X3[k] + m4[k] * us[k];
  }
  mxm_4(S2s, s->G2T, X2);
  mxm_4(S2z, s->G2T, X4);
  mxm_4(G, S1s, X1);
  mxm_4(G, S1z, X3);
  for (int k = 0; k < 25; ++k) {
    ls[k] = ls[k] + X1[k] + X2[k];
    lz[k] = X3[k] + X4[k];
  }
  if (axis) {
    vec5 uz0, V1, V2, V3, V4, w1, w2, w3, t;
    for (int j = 0; j < 5; ++j) {
      uz0[j] = A(uz, 0, j);
      w1[j] = (REAL)M0(AXG_M0_W1)[j];
      w2[j] = (REAL)M0(AXG_M0_W2)[j];
      w3[j] = (REAL)M0(AXG_M0_W3)[j];
    }
    vxm_4(s->G0, us, V1);
    vxm_4(uz0, s->G2, V2);
    for (int j = 0; j < 5; ++j) V4[j] = w1[j] * V1[j] + w3[j] * V2[j];
    vxm_4(s->G0, uz, V3);
    for (int j = 0; j < 5; ++j) V4[j] = V4[j] + w2[j] * V3[j];
    for (int j = 0; j < 5; ++j) t[j] = w2[j] * V1[j];
    outerprod_4(s->G0, t, X2);
    for (int j = 0; j < 5; ++j) V2[j] = w3[j] * V1[j];
    vxm_4(V2, s->G2T, V1);
    for (int j = 0; j < 5; ++j) A(X2, 0, j) = A(X2, 0, j) + V1[j];
    outerprod_4(s->G0, V4, X1);
    for (int k = 0; k < 25; ++k) {
      ls[k] = ls[k] + X1[k];
      lz[k] = X2[k] + lz[k];
    }
  }
  memcpy(out_s, ls, sizeof ls);
  memcpy(out_z, lz, sizeof lz);
}

/* glob_stiffness_di_4, SOLVER/stiffness_di.f90:60-256 */
static void stiff_di_el(const axg_mesh_desc *d, const spec *s, int64_t e, int axis,
                        const REAL *u1_, const REAL *u2_, const REAL *u3_,
                        REAL *o1, REAL *o2, REAL *o3) {
  const int64_t off = 25 * e, off0 = 5 * e;
  mat5 u1, u2, u3, X1, X2, X3, X4, X5, X6, X7, X8;
  mat5 ls2, ls3, s1p, s1m, s2p, s2m, S1z, S2z, l1, l2, l3;
  mat5 m1, m2, m3, m4, m5, m6, m7, m8, mw1, mw2, mw3;
  mat5 m11s, m21s, m41s, m12s, m22s, m42s, m13s, m23s, m33s, m43s, m11z, m21z, m41z;
  memcpy(u1, u1_, sizeof u1);
  memcpy(u2, u2_, sizeof u2);
  memcpy(u3, u3_, sizeof u3);
  load_mat(m1, MS(AXG_M_1)); load_mat(m2, MS(AXG_M_2)); load_mat(m3, MS(AXG_M_3));
  load_mat(m4, MS(AXG_M_4)); load_mat(m5, MS(AXG_M_5)); load_mat(m6, MS(AXG_M_6));
  load_mat(m7, MS(AXG_M_7)); load_mat(m8, MS(AXG_M_8));
  load_mat(mw1, MS(AXG_M_W1)); load_mat(mw2, MS(AXG_M_W2)); load_mat(mw3, MS(AXG_M_W3));
  load_mat(m11s, MS(AXG_M11S)); load_mat(m21s, MS(AXG_M21S)); load_mat(m41s, MS(AXG_M41S));
  load_mat(m12s, MS(AXG_M12S)); load_mat(m22s, MS(AXG_M22S)); load_mat(m42s, MS(AXG_M42S));
  load_mat(m13s, MS(AXG_M13S));
  load_mat(m23s, MS(AXG_M32S)); /* m23sl = M32s, SOLVER/stiffness_di.f90:122 */
  load_mat(m33s, MS(AXG_M33S)); load_mat(m43s, MS(AXG_M43S));
  load_mat(m11z, MS(AXG_M11Z)); load_mat(m21z, MS(AXG_M21Z)); load_mat(m41z, MS(AXG_M41Z));

  const REAL *GT = axis ? s->G1T : s->G2T;
  const REAL *G = axis ? s->G1 : s->G2;
  mxm_4(u1, s->G2, X4);
  mxm_4(u2, s->G2, X5);
  mxm_4(u3, s->G2, X6);
  mxm_4(GT, u1, X1);
  mxm_4(GT, u2, X2);
  mxm_4(GT, u3, X3);
  for (int k = 0; k < 25; ++k) {
    X7[k] = X1[k] + X2[k];
    X8[k] = X4[k] + X5[k];
  }
  for (int k = 0; k < 25; ++k) {
    ls2[k] = m8[k] * X6[k] + m7[k] * X3[k] + m1[k] * X1[k] + m5[k] * X2[k] + m2[k] * X4[k] +
             m6[k] * X5[k] + mw1[k] * u2[k] + mw2[k] * u3[k];
    ls3[k] = m4[k] * X4[k] - m4[k] * X5[k] + m3[k] * X1[k] - m3[k] * X2[k] + mw2[k] * u2[k] +
             mw3[k] * u3[k];
    REAL c1 = m13s[k] * X6[k], c2 = m23s[k] * X3[k], c3 = m3[k] * u3[k];
    s1p[k] = c1 + c2 + c3 + m11s[k] * X4[k] + m21s[k] * X1[k] + m12s[k] * X5[k] + m22s[k] * X2[k] +
             m1[k] * u2[k];
    s1m[k] = c1 + c2 - c3 + m11s[k] * X5[k] + m21s[k] * X2[k] + m12s[k] * X4[k] + m22s[k] * X1[k] +
             m5[k] * u2[k];
    c1 = m33s[k] * X3[k];
    c2 = m43s[k] * X6[k];
    c3 = m4[k] * u3[k];
    s2p[k] = c1 + c2 + c3 + m11s[k] * X1[k] + m41s[k] * X4[k] + m12s[k] * X2[k] + m42s[k] * X5[k] +
             m2[k] * u2[k];
    s2m[k] = c1 + c2 - c3 + m11s[k] * X2[k] + m41s[k] * X5[k] + m12s[k] * X1[k] + m42s[k] * X4[k] +
             m6[k] * u2[k];
    S1z[k] = m33s[k] * X8[k] + m23s[k] * X7[k] + m11z[k] * X6[k] + m21z[k] * X3[k] + m7[k] * u2[k];
    S2z[k] = m13s[k] * X7[k] + m43s[k] * X8[k] + m11z[k] * X3[k] + m41z[k] * X6[k] + m8[k] * u2[k];
  }
  mxm_4(G, s1p, X1);
  mxm_4(G, s1m, X3);
  mxm_4(G, S1z, X5);
  mxm_4(s2p, s->G2T, X2);
  mxm_4(s2m, s->G2T, X4);
  mxm_4(S2z, s->G2T, X6);
  for (int k = 0; k < 25; ++k) {
    l1[k] = X1[k] + X2[k];
    l2[k] = X3[k] + X4[k] + ls2[k];
    l3[k] = X5[k] + X6[k] + ls3[k];
  }
  if (axis) {
    vec5 w[11], u10, u20, V1, V2, V3, V4, V5, t;
    for (int j = 0; j < 5; ++j) {
      u10[j] = A(u1, 0, j);
      u20[j] = A(u2, 0, j);
    }
    const int used[9] = {1, 2, 3, 4, 6, 7, 8, 9, 10};
    for (int q = 0; q < 9; ++q)
      for (int j = 0; j < 5; ++j) w[used[q]][j] = (REAL)M0(AXG_M0_W1 + used[q] - 1)[j];
    vxm_4(s->G0, u1, V1);
    vxm_4(s->G0, u2, V2);
    vxm_4(s->G0, u3, V3);
    vxm_4(u10, s->G2, V4);
    vxm_4(u20, s->G2, V5);
    for (int j = 0; j < 5; ++j) t[j] = w[1][j] * V2[j] + w[3][j] * V3[j];
    outerprod_4(s->G0, t, s1p);
    for (int j = 0; j < 5; ++j)
      t[j] = w[1][j] * V1[j] + (w[2][j] + w[6][j]) * V4[j] + w[9][j] * V2[j] + w[10][j] * V3[j];
    outerprod_4(s->G0, t, s1m);
    for (int j = 0; j < 5; ++j)
      t[j] = w[3][j] * V1[j] + (w[4][j] + w[8][j]) * V4[j] + w[7][j] * V3[j] + w[10][j] * V2[j];
    outerprod_4(s->G0, t, S1z);
    for (int j = 0; j < 5; ++j) V4[j] = (w[2][j] + w[6][j]) * V2[j] + (w[4][j] + w[8][j]) * V3[j];
    vxm_4(V4, s->G2T, V1);
    for (int j = 0; j < 5; ++j) A(s1p, 0, j) = A(s1p, 0, j) + V1[j];
    for (int k = 0; k < 25; ++k) {
      l1[k] = l1[k] + s1p[k];
      l2[k] = l2[k] + s1m[k];
      l3[k] = l3[k] + S1z[k];
    }
  }
  memcpy(o1, l1, sizeof l1);
  memcpy(o2, l2, sizeof l2);
  memcpy(o3, l3, sizeof l3);
}

/* glob_stiffness_quad_4, SOLVER/stiffness_quad.f90:238-414 */
static void stiff_quad_el(const axg_mesh_desc *d, const spec *s, int64_t e, int axis,
                          const REAL *us_, const REAL *up_, const REAL *uz_,
                          REAL *o1, REAL *o2, REAL *o3) {
  const int64_t off = 25 * e, off0 = 5 * e;
  mat5 us, up, uz, X1, X2, X3, X4, X5, X6, ls, lp, lz, S1s, S2s, S1z, S2z, S1p, S2p;
  mat5 m1, m2, m3, m4, m5, m6, m7, m8, mw1, mw2, mw3, mw4, mw5;
  mat5 m11s, m21s, m41s, m12s, m22s, m32s, m42s, m11z, m21z, m41z, m1p, m2p, m4p;
  memcpy(us, us_, sizeof us);
  memcpy(up, up_, sizeof up);
  memcpy(uz, uz_, sizeof uz);
  load_mat(m1, MS(AXG_M_1)); load_mat(m2, MS(AXG_M_2)); load_mat(m3, MS(AXG_M_3));
  load_mat(m4, MS(AXG_M_4)); load_mat(m5, MS(AXG_M_5)); load_mat(m6, MS(AXG_M_6));
  load_mat(m7, MS(AXG_M_7)); load_mat(m8, MS(AXG_M_8));
  load_mat(mw1, MS(AXG_M_W1)); load_mat(mw2, MS(AXG_M_W2)); load_mat(mw3, MS(AXG_M_W3));
  load_mat(mw4, MS(AXG_M_W4)); load_mat(mw5, MS(AXG_M_W5));
  load_mat(m11s, MS(AXG_M11S)); load_mat(m21s, MS(AXG_M21S)); load_mat(m41s, MS(AXG_M41S));
  load_mat(m12s, MS(AXG_M12S)); load_mat(m22s, MS(AXG_M22S)); load_mat(m32s, MS(AXG_M32S));
  load_mat(m42s, MS(AXG_M42S));
  load_mat(m11z, MS(AXG_M11Z)); load_mat(m21z, MS(AXG_M21Z)); load_mat(m41z, MS(AXG_M41Z));
  load_mat(m1p, MS(AXG_M1PHI)); load_mat(m2p, MS(AXG_M2PHI)); load_mat(m4p, MS(AXG_M4PHI));

  const REAL *GT = axis ? s->G1T : s->G2T;
  const REAL *G = axis ? s->G1 : s->G2;
  mxm_4(GT, us, X1);
  mxm_4(GT, up, X2);
  mxm_4(GT, uz, X3);
  mxm_4(us, s->G2, X4);
  mxm_4(up, s->G2, X5);
  mxm_4(uz, s->G2, X6);
  for (int k = 0; k < 25; ++k) {
    REAL c1 = m2[k] * X4[k], c2 = m1[k] * X1[k], c3 = m6[k] * X5[k];
    REAL c4 = m5[k] * X2[k], c5 = m4[k] * X6[k], c6 = m3[k] * X3[k];
    ls[k] = c1 + c2 + 2 * (c3 + c4) + c5 + c6 + mw1[k] * us[k] + mw2[k] * up[k] + 2 * mw3[k] * uz[k];
    lp[k] = -2 * (c1 + c2 + c5 + c6) - (c3 + c4) + mw2[k] * us[k] + mw4[k] * up[k] - mw3[k] * uz[k];
    lz[k] = 2 * (m8[k] * X5[k] + m7[k] * X2[k]) + mw3[k] * (2 * us[k] - up[k]) + mw5[k] * uz[k];
    REAL usm = us[k] - 2 * up[k];
    S1s[k] = m11s[k] * X4[k] + m21s[k] * X1[k] + m12s[k] * X6[k] + m22s[k] * X3[k] + m1[k] * usm;
    S2s[k] = m11s[k] * X1[k] + m41s[k] * X4[k] + m32s[k] * X3[k] + m42s[k] * X6[k] + m2[k] * usm;
    S1z[k] = m11z[k] * X6[k] + m21z[k] * X3[k] + m32s[k] * X4[k] + m22s[k] * X1[k] + m3[k] * usm;
    S2z[k] = m11z[k] * X3[k] + m41z[k] * X6[k] + m12s[k] * X1[k] + m42s[k] * X4[k] + m4[k] * usm;
    REAL ups = 2 * us[k] - up[k];
    S1p[k] = m1p[k] * X5[k] + m2p[k] * X2[k] + m5[k] * ups + 2 * m7[k] * uz[k];
    S2p[k] = m1p[k] * X2[k] + m4p[k] * X5[k] + m6[k] * ups + 2 * m8[k] * uz[k];
  }
  mxm_4(S2s, s->G2T, X2);
  mxm_4(S2p, s->G2T, X4);
  mxm_4(S2z, s->G2T, X6);
  mxm_4(G, S1s, X1);
  mxm_4(G, S1p, X3);
  mxm_4(G, S1z, X5);
  for (int k = 0; k < 25; ++k) {
    ls[k] = ls[k] + X1[k] + X2[k];
    lp[k] = lp[k] + X3[k] + X4[k];
    lz[k] = lz[k] + X5[k] + X6[k];
  }
  if (axis) {
    vec5 w1, w2, w3, w4, w5, w6, V1, V2, V3, t;
    for (int j = 0; j < 5; ++j) {
      w1[j] = (REAL)M0(AXG_M0_W1)[j]; w2[j] = (REAL)M0(AXG_M0_W2)[j];
      w3[j] = (REAL)M0(AXG_M0_W3)[j]; w4[j] = (REAL)M0(AXG_M0_W4)[j];
      w5[j] = (REAL)M0(AXG_M0_W5)[j]; w6[j] = (REAL)M0(AXG_M0_W6)[j];
    }
    vxm_4(s->G0, us, V1);
    vxm_4(s->G0, up, V2);
    vxm_4(s->G0, uz, V3);
    for (int j = 0; j < 5; ++j) t[j] = w1[j] * V1[j] + w2[j] * V2[j] + w3[j] * V3[j];
    outerprod_4(s->G0, t, S1s);
    for (int j = 0; j < 5; ++j) t[j] = w2[j] * V1[j] + w4[j] * V2[j] + w5[j] * V3[j];
    outerprod_4(s->G0, t, S1p);
    for (int j = 0; j < 5; ++j) t[j] = w3[j] * V1[j] + w5[j] * V2[j] + w6[j] * V3[j];
    outerprod_4(s->G0, t, S1z);
    for (int k = 0; k < 25; ++k) {
      ls[k] = ls[k] + S1s[k];
      lp[k] = lp[k] + S1p[k];
      lz[k] = lz[k] + S1z[k];
    }
  }
  memcpy(o1, ls, sizeof ls);
  memcpy(o2, lp, sizeof lp);
  memcpy(o3, lz, sizeof lz);
}

/* glob_stiffness_{mono,di,quad} over all solid elements, element-local in/out
 * u(0:4,0:4,nel_solid,3) -> out(0:4,0:4,nel_solid,3).  Monopole leaves
 * component 2 at zero (the reference leaves it undefined). */
void ORC(stiffness_solid)(const axg_mesh_desc *d, const REAL *u, REAL *out) {
  spec s;
  load_spec(d, &s);
  const int64_t ne = d->nel_solid, cs = 25 * ne;
  unsigned char *ax = axis_flags(d->nel_solid, d->naxel_solid, d->ax_el_solid);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e) {
    const REAL *u1 = u + 25 * e, *u2 = u1 + cs, *u3 = u2 + cs;
    REAL *o1 = out + 25 * e, *o2 = o1 + cs, *o3 = o2 + cs;
    if (d->src_type == AXG_MONOPOLE) {
      stiff_mono_el(d, &s, e, ax[e], u1, u3, o1, o3);
      for (int k = 0; k < 25; ++k) o2[k] = 0;
    } else if (d->src_type == AXG_DIPOLE) {
      stiff_di_el(d, &s, e, ax[e], u1, u2, u3, o1, o2, o3);
    } else {
      stiff_quad_el(d, &s, e, ax[e], u1, u2, u3, o1, o2, o3);
    }
  }
  free(ax);
}

/* glob_fluid_stiffness_4, SOLVER/stiffness_fluid.f90:139-216 */
void ORC(stiffness_fluid)(const axg_mesh_desc *d, const REAL *chi, REAL *out) {
  spec s;
  load_spec(d, &s);
  unsigned char *ax = axis_flags(d->nel_fluid, d->naxel_fluid, d->ax_el_fluid);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < d->nel_fluid; ++e) {
    const int64_t off = 25 * e;
    mat5 c, X1, X2, S1, S2, m1, m2, m4, loc;
    memcpy(c, chi + off, sizeof c);
    load_mat(m1, d->m_fluid[AXG_M1CHI] + off);
    load_mat(m2, d->m_fluid[AXG_M2CHI] + off);
    load_mat(m4, d->m_fluid[AXG_M4CHI] + off);
    mxm_4(ax[e] ? s.G1T : s.G2T, c, X1);
    mxm_4(c, s.G2, X2);
    for (int k = 0; k < 25; ++k) {
      S1[k] = m1[k] * X2[k] + m2[k] * X1[k];
      S2[k] = m1[k] * X1[k] + m4[k] * X2[k];
    }
    mxm_4(ax[e] ? s.G1 : s.G2, S1, X1);
    mxm_4(S2, s.G2T, X2);
    for (int k = 0; k < 25; ++k) loc[k] = X1[k] + X2[k];
    if (d->src_type != AXG_MONOPOLE) {
      const float *mw = d->m_fluid[AXG_M_W_FL] + off;
      for (int k = 0; k < 25; ++k) loc[k] = loc[k] + (REAL)mw[k] * c[k];
      if (ax[e]) {
        vec5 V1, t;
        vxm_4(s.G0, c, V1);
        for (int j = 0; j < 5; ++j) t[j] = (REAL)d->m0_w_fl[5 * e + j] * V1[j];
        outerprod_4(s.G0, t, c);
        for (int k = 0; k < 25; ++k) loc[k] = loc[k] + c[k];
      }
    }
    memcpy(out + off, loc, sizeof loc);
  }
  free(ax);
}

/* ------------------------------------------------------- attenuation (cg4) */

#define CG(arr, e) ((arr) + 4 * (e))
static void load4(REAL *dst, const float *src) {
  for (int k = 0; k < 4; ++k) dst[k] = (REAL)src[k];
}

/* glob_anel_stiffness_{mono,di,quad}_cg4: subtracts the memory-variable
 * stress divergence.  R = memory_var_cg4(1:4,6,n_sls,nel_solid). */
void ORC(anel_stiffness_cg4)(const axg_mesh_desc *d, const REAL *R, REAL *gs) {
  spec s;
  load_spec(d, &s);
  const int64_t ne = d->nel_solid, cs = 25 * ne;
  const int nsls = d->n_sls;
  unsigned char *ax = axis_flags(d->nel_solid, d->naxel_solid, d->ax_el_solid);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e) {
    REAL yl[4], vse[4], vsx[4], vze[4], vzx[4], r[7][4];
    load4(yl, CG(d->Y_cg4, e));
    load4(vse, CG(d->V_s_eta_cg4, e));
    load4(vsx, CG(d->V_s_xi_cg4, e));
    load4(vze, CG(d->V_z_eta_cg4, e));
    load4(vzx, CG(d->V_z_xi_cg4, e));
    for (int c = 1; c <= 6; ++c)
      for (int k = 0; k < 4; ++k) r[c][k] = 0;
    for (int j = 0; j < nsls; ++j)
      for (int c = 1; c <= 6; ++c)
        for (int k = 0; k < 4; ++k)
          r[c][k] = r[c][k] + R[k + 4 * ((c - 1) + 6 * (j + (int64_t)nsls * e))];
    const REAL *G = ax[e] ? s.G1 : s.G2;
    REAL S1a[4], S2a[4], S1b[4], S2b[4], S1z[4], S2z[4];
    mat5 X1, X2, X3, X4, X5, X6, la, lb, lz;
    REAL *g1 = gs + 25 * e, *g2 = g1 + cs, *g3 = g2 + cs;
    if (d->src_type == AXG_MONOPOLE) {
      for (int k = 0; k < 4; ++k) {
        S1a[k] = vze[k] * r[1][k] + vse[k] * r[5][k];
        S2a[k] = vzx[k] * r[1][k] + vsx[k] * r[5][k];
        S1z[k] = vze[k] * r[5][k] + vse[k] * r[3][k];
        S2z[k] = vzx[k] * r[5][k] + vsx[k] * r[3][k];
      }
      mxm_cg4_sparse_b(G, S1a, X1);
      mxm_cg4_sparse_b(G, S1z, X3);
      mxm_cg4_sparse_a(S2a, s.G2T, X2);
      mxm_cg4_sparse_a(S2z, s.G2T, X4);
      for (int k = 0; k < 25; ++k) {
        la[k] = X1[k] + X2[k];
        lz[k] = X3[k] + X4[k];
      }
      A(la, 1, 1) = A(la, 1, 1) + yl[0] * r[2][0];
      A(la, 1, 3) = A(la, 1, 3) + yl[1] * r[2][1];
      A(la, 3, 1) = A(la, 3, 1) + yl[2] * r[2][2];
      A(la, 3, 3) = A(la, 3, 3) + yl[3] * r[2][3];
      for (int k = 0; k < 25; ++k) {
        g1[k] = g1[k] - la[k];
        g3[k] = g3[k] - lz[k];
      }
    } else {
      const int di = d->src_type == AXG_DIPOLE;
      for (int k = 0; k < 4; ++k) {
        if (di) {
          S1a[k] = vze[k] * (r[1][k] - r[6][k]) + vse[k] * (r[5][k] - r[4][k]);
          S2a[k] = vzx[k] * (r[1][k] - r[6][k]) + vsx[k] * (r[5][k] - r[4][k]);
          S1b[k] = vze[k] * (r[1][k] + r[6][k]) + vse[k] * (r[5][k] + r[4][k]);
          S2b[k] = vzx[k] * (r[1][k] + r[6][k]) + vsx[k] * (r[5][k] + r[4][k]);
        } else {
          S1a[k] = vze[k] * r[1][k] + vse[k] * r[5][k];
          S2a[k] = vzx[k] * r[1][k] + vsx[k] * r[5][k];
          S1b[k] = vze[k] * r[6][k] + vse[k] * r[4][k];
          S2b[k] = vzx[k] * r[6][k] + vsx[k] * r[4][k];
        }
        S1z[k] = vze[k] * r[5][k] + vse[k] * r[3][k];
        S2z[k] = vzx[k] * r[5][k] + vsx[k] * r[3][k];
      }
      mxm_cg4_sparse_b(G, S1a, X1);
      mxm_cg4_sparse_b(G, S1b, X3);
      mxm_cg4_sparse_b(G, S1z, X5);
      mxm_cg4_sparse_a(S2a, s.G2T, X2);
      mxm_cg4_sparse_a(S2b, s.G2T, X4);
      mxm_cg4_sparse_a(S2z, s.G2T, X6);
      const int pi_[4] = {1, 1, 3, 3}, pj_[4] = {1, 3, 1, 3};
      if (di) {
        for (int k = 0; k < 25; ++k) {
          la[k] = X1[k] + X2[k];
          lb[k] = X3[k] + X4[k];
          lz[k] = X5[k] + X6[k];
        }
        for (int p = 0; p < 4; ++p) {
          A(lb, pi_[p], pj_[p]) = A(lb, pi_[p], pj_[p]) + 2 * yl[p] * (r[2][p] - r[6][p]);
          A(lz, pi_[p], pj_[p]) = A(lz, pi_[p], pj_[p]) - yl[p] * r[4][p];
        }
      } else {
        for (int k = 0; k < 25; ++k) {
          la[k] = X1[k] + X2[k];
          lb[k] = -X3[k] - X4[k];
          lz[k] = X5[k] + X6[k];
        }
        for (int p = 0; p < 4; ++p) {
          A(la, pi_[p], pj_[p]) = A(la, pi_[p], pj_[p]) + yl[p] * (r[2][p] - 2 * r[6][p]);
          A(lb, pi_[p], pj_[p]) = A(lb, pi_[p], pj_[p]) + yl[p] * (r[6][p] - 2 * r[2][p]);
          A(lz, pi_[p], pj_[p]) = A(lz, pi_[p], pj_[p]) - 2 * yl[p] * r[4][p];
        }
      }
      for (int k = 0; k < 25; ++k) {
        g1[k] = g1[k] - la[k];
        g2[k] = g2[k] - lb[k];
        g3[k] = g3[k] - lz[k];
      }
    }
  }
  free(ax);
}

/* axisym_gradient_solid_el_cg4: grad(:,1) = d/ds, grad(:,2) = d/dz at cg4 points */
static void gradient_cg4(const axg_mesh_desc *d, const spec *s, int64_t e, int axis,
                         const REAL *f, REAL g[2][4]) {
  REAL dzdeta[4], dzdxi[4], dsdeta[4], dsdxi[4], m1[4], m2[4];
  load4(dzdeta, CG(d->DzDeta_over_J_sol_cg4, e));
  load4(dzdxi, CG(d->DzDxi_over_J_sol_cg4, e));
  load4(dsdeta, CG(d->DsDeta_over_J_sol_cg4, e));
  load4(dsdxi, CG(d->DsDxi_over_J_sol_cg4, e));
  mxm_cg4_sparse_c(axis ? s->G1T : s->G2T, f, m1);
  mxm_cg4_sparse_c(f, s->G2, m2);
  for (int k = 0; k < 4; ++k) {
    g[0][k] = dzdeta[k] * m1[k] + dzdxi[k] * m2[k];
    g[1][k] = dsdeta[k] * m1[k] + dsdxi[k] * m2[k];
  }
}

/* f_over_s_solid_el_cg4 */
static void f_over_s_cg4(const axg_mesh_desc *d, int64_t e, const REAL *f, REAL *o) {
  const float *is = d->inv_s_solid + 25 * e;
  o[0] = (REAL)is[1 + 5 * 1] * A(f, 1, 1);
  o[1] = (REAL)is[1 + 5 * 3] * A(f, 1, 3);
  o[2] = (REAL)is[3 + 5 * 1] * A(f, 3, 1);
  o[3] = (REAL)is[3 + 5 * 3] * A(f, 3, 3);
}

/* compute_strain_att_el_cg4, SOLVER/attenuation.f90:471-535: grad_u(1:4,6) in
 * Voigt order; u = disp(:,:,iel,1:3) element-local. */
static void strain_cg4(const axg_mesh_desc *d, const spec *s, int64_t e, int axis,
                       const REAL *u1, const REAL *u2, const REAL *u3, REAL gu[7][4]) {
  REAL b1[2][4], b2[2][4], t[4], t2[4];
  mat5 tmp;
  for (int c = 1; c <= 6; ++c)
    for (int k = 0; k < 4; ++k) gu[c][k] = 0;
  if (d->src_type == AXG_DIPOLE) {
    for (int k = 0; k < 25; ++k) tmp[k] = u1[k] + u2[k];
    gradient_cg4(d, s, e, axis, tmp, b1);
  } else {
    gradient_cg4(d, s, e, axis, u1, b1);
  }
  gradient_cg4(d, s, e, axis, u3, b2);
  for (int k = 0; k < 4; ++k) {
    gu[1][k] = b1[0][k];
    gu[3][k] = b2[1][k];
    gu[5][k] = b1[1][k] + b2[0][k];
  }
  if (d->src_type == AXG_MONOPOLE) {
    f_over_s_cg4(d, e, u1, t);
    for (int k = 0; k < 4; ++k) gu[2][k] = t[k];
  } else if (d->src_type == AXG_DIPOLE) {
    f_over_s_cg4(d, e, u2, t);
    for (int k = 0; k < 4; ++k) gu[2][k] = 2 * t[k];
    for (int k = 0; k < 25; ++k) tmp[k] = u1[k] - u2[k];
    gradient_cg4(d, s, e, axis, tmp, b1);
    f_over_s_cg4(d, e, u3, t);
    for (int k = 0; k < 4; ++k) {
      gu[4][k] = -t[k] - b1[1][k];
      gu[6][k] = -gu[2][k] - b1[0][k];
    }
  } else {
    for (int k = 0; k < 25; ++k) tmp[k] = u1[k] - 2 * u2[k];
    f_over_s_cg4(d, e, tmp, t);
    for (int k = 0; k < 4; ++k) gu[2][k] = t[k];
    gradient_cg4(d, s, e, axis, u2, b1);
    f_over_s_cg4(d, e, u3, t);
    for (int k = 0; k < 25; ++k) tmp[k] = u2[k] - 2 * u1[k];
    f_over_s_cg4(d, e, tmp, t2);
    for (int k = 0; k < 4; ++k) {
      gu[4][k] = -2 * t[k] - b1[1][k];
      gu[6][k] = t2[k] - b1[0][k];
    }
  }
}

/* fast_correct, SOLVER/attenuation.f90:1139-1155 */
static void fast_correct(const double *y, double *yp, int n) {
  double dy = 1 + .5 * y[0];
  double prev = dy;
  yp[0] = y[0] * dy;
  for (int k = 1; k < n; ++k) {
    dy = prev + (prev - .5) * y[k - 1] + .5 * y[k];
    yp[k] = y[k] * dy;
    prev = dy;
  }
}

/* a_j = yp_j / sum(yp_j) with yp_j = y_j / Q (optionally corrected) */
void ORC(sls_weights)(const axg_mesh_desc *d, double Q, double *a) {
  double y[32], yp[32], sum = 0;
  const int n = d->n_sls;
  for (int j = 0; j < n; ++j) y[j] = d->y_j_attenuation[j] / Q;
  if (d->do_corr_lowq)
    fast_correct(y, yp, n);
  else
    for (int j = 0; j < n; ++j) yp[j] = y[j];
  for (int j = 0; j < n; ++j) sum += yp[j];
  for (int j = 0; j < n; ++j) a[j] = yp[j] / sum;
}

/* time_step_memvars_cg4, SOLVER/attenuation.f90:81-202.
 * memvar(1:4,6,n_sls,nel), src_tr_tm1(1:4,nel), src_dev_tm1(1:4,6,nel). */
void ORC(time_step_memvars_cg4)(const axg_mesh_desc *d, REAL *memvar, const REAL *disp,
                                REAL *src_tr_tm1_glob, REAL *src_dev_tm1_glob) {
  spec s;
  load_spec(d, &s);
  const int64_t ne = d->nel_solid, cs = 25 * ne;
  const int nsls = d->n_sls;
  const double third = 1.0 / 3.0;
  unsigned char *ax = axis_flags(d->nel_solid, d->naxel_solid, d->ax_el_solid);
  /* elements are independent; each thread keeps its own cache of the SLS
   * weights of the last Q value it met (a deterministic function of Q) */
#pragma omp parallel
  {
  double a_mu[32], a_ka[32];
  double Qmu_last = NAN, Qka_last = NAN;
#pragma omp for schedule(static)
  for (int64_t e = 0; e < ne; ++e) {
    REAL gu[7][4];
    strain_cg4(d, &s, e, ax[e], disp + 25 * e, disp + cs + 25 * e, disp + 2 * cs + 25 * e, gu);
    if (!((double)d->Q_mu[e] == Qmu_last)) {
      Qmu_last = d->Q_mu[e];
      ORC(sls_weights)(d, Qmu_last, a_mu);
    }
    if (!((double)d->Q_kappa[e] == Qka_last)) {
      Qka_last = d->Q_kappa[e];
      ORC(sls_weights)(d, Qka_last, a_ka);
    }
    REAL tr[4], src_tr[4], src_dev[7][4];
    for (int k = 0; k < 4; ++k) tr[k] = gu[1][k] + gu[2][k] + gu[3][k];
    const float *dmu = CG(d->delta_mu_cg4, e), *dka = CG(d->delta_kappa_cg4, e);
    for (int c = 1; c <= 6; ++c)
      for (int k = 0; k < 4; ++k) src_dev[c][k] = 0;
    for (int k = 0; k < 4; ++k) {
      REAL dm = (REAL)dmu[k];
      src_tr[k] = (REAL)dka[k] * tr[k];
      for (int c = 1; c <= 3; ++c)
        src_dev[c][k] = (REAL)((double)(dm * 2) * ((double)gu[c][k] - (double)tr[k] * third));
      src_dev[5][k] = dm * gu[5][k];
      if (d->src_type != AXG_MONOPOLE) {
        src_dev[4][k] = dm * gu[4][k];
        src_dev[6][k] = dm * gu[6][k];
      }
    }
    REAL *trm1 = src_tr_tm1_glob + 4 * e, *devm1 = src_dev_tm1_glob + 24 * e;
    for (int j = 0; j < nsls; ++j) {
      const double ft = d->ts_fac_t[j], ftm1 = d->ts_fac_tm1[j], ex = d->exp_w_j_deltat[j];
      REAL *R = memvar + 4 * 6 * (j + (int64_t)nsls * e);
      for (int k = 0; k < 4; ++k) {
        REAL trb = (REAL)(ft * a_ka[j] * src_tr[k] + ftm1 * a_ka[j] * trm1[k]);
        REAL db[7];
        for (int c = 1; c <= 6; ++c)
          db[c] = (REAL)(ft * a_mu[j] * src_dev[c][k] + ftm1 * a_mu[j] * devm1[k + 4 * (c - 1)]);
        R[k + 4 * 0] = (REAL)(ex * R[k + 4 * 0] + db[1] + trb);
        R[k + 4 * 1] = (REAL)(ex * R[k + 4 * 1] + db[2] + trb);
        R[k + 4 * 2] = (REAL)(ex * R[k + 4 * 2] + db[3] + trb);
        R[k + 4 * 4] = (REAL)(ex * R[k + 4 * 4] + db[5]);
        if (d->src_type != AXG_MONOPOLE) {
          R[k + 4 * 3] = (REAL)(ex * R[k + 4 * 3] + db[4]);
          R[k + 4 * 5] = (REAL)(ex * R[k + 4 * 5] + db[6]);
        }
      }
    }
    for (int k = 0; k < 4; ++k) {
      trm1[k] = src_tr[k];
      for (int c = 1; c <= 6; ++c) devm1[k + 4 * (c - 1)] = src_dev[c][k];
    }
  }
  }
  free(ax);
}

/* axisym_gradient_solid / _fluid on one element
 * (SOLVER/pointwise_derivatives.f90:329-365, 509-545):
 *   mxm1 = G1T f (axial element) or G2T f, mxm2 = f G2,
 *   d/ds = dzdeta * mxm1 + dzdxi * mxm2,  d/dz = dsdeta * mxm1 + dsdxi * mxm2
 * (the reference's names of the mapping terms). */
typedef struct pw_el {
  const float *dsdeta, *dzdeta, *dsdxi, *dzdxi, *inv_s;
} pw_el;

static void grad_el(const spec *s, int axis, const pw_el *w, const REAL *f, REAL *gs, REAL *gz) {
  mat5 m1, m2;
  mxm_4(axis ? s->G1T : s->G2T, f, m1);
  mxm_4(f, s->G2, m2);
  for (int k = 0; k < 25; ++k) {
    gs[k] = (REAL)w->dzdeta[k] * m1[k] + (REAL)w->dzdxi[k] * m2[k];
    gz[k] = (REAL)w->dsdeta[k] * m1[k] + (REAL)w->dsdxi[k] * m2[k];
  }
}

/* f_over_s_solid / _fluid on one element (SOLVER/pointwise_derivatives.f90:
 * 130-178): inv_s * f, and at the axis (ipol = 0 of an axial element)
 * L'Hospital's f/s = df/ds (dsdf_*_allaxis, always with G1T, :480-505). */
static void f_over_s_el(const spec *s, int axis, const pw_el *w, const REAL *f, REAL *o) {
  for (int k = 0; k < 25; ++k) o[k] = (REAL)w->inv_s[k] * f[k];
  if (!axis) return;
  mat5 m1, m2;
  mxm_4(s->G1T, f, m1);
  mxm_4(f, s->G2, m2);
  for (int j = 0; j < 5; ++j) o[5 * j] = (REAL)w->dzdeta[5 * j] * m1[5 * j] + (REAL)w->dzdxi[5 * j] * m2[5 * j];
}

/* ------------------------------------------------ attenuation (full, npol = 4) */

/* The not coarse-grained variant (att_coarse_grained = .false.): memory
 * variables at all 25 GLL points.  Arrays per point (0:4,0:4,nel_solid):
 * delta_mu, delta_kappa, Y, V_*; per axial element (0:4,nel_solid): Y0,
 * V0_*; the strain uses the data_pointwise mapping terms and inv_s_solid. */

/* the solid's data_pointwise terms of element e (the descriptor's copies) */
static void pw_of(const axg_mesh_desc *d, int64_t e, pw_el *w) {
  w->dsdeta = d->DsDeta_over_J_sol + 25 * e;
  w->dzdeta = d->DzDeta_over_J_sol + 25 * e;
  w->dsdxi = d->DsDxi_over_J_sol + 25 * e;
  w->dzdxi = d->DzDxi_over_J_sol + 25 * e;
  w->inv_s = d->inv_s_solid + 25 * e;
}

/* compute_strain_att_el_4, SOLVER/attenuation.f90:542-606: grad_u(0:4,0:4,6)
 * in Voigt order, from axisym_gradient_solid_el_4 and f_over_s_solid_el_4
 * (SOLVER/pointwise_derivatives.f90:104-126, 252-286). */
static void strain_att_4(const axg_mesh_desc *d, const spec *s, int64_t e, int axis, const REAL *u1,
                         const REAL *u2, const REAL *u3, REAL gu[7][25]) {
  pw_el w;
  pw_of(d, e, &w);
  mat5 b1s, b1z, b2s, b2z, tmp, t, t2;
  for (int c = 1; c <= 6; ++c)
    for (int k = 0; k < 25; ++k) gu[c][k] = 0;
  if (d->src_type == AXG_DIPOLE) {
    for (int k = 0; k < 25; ++k) tmp[k] = u1[k] + u2[k];
    grad_el(s, axis, &w, tmp, b1s, b1z);
  } else {
    grad_el(s, axis, &w, u1, b1s, b1z);
  }
  grad_el(s, axis, &w, u3, b2s, b2z);
  for (int k = 0; k < 25; ++k) {
    gu[1][k] = b1s[k];
    gu[3][k] = b2z[k];
    gu[5][k] = b1z[k] + b2s[k];
  }
  if (d->src_type == AXG_MONOPOLE) {
    f_over_s_el(s, axis, &w, u1, t);
    for (int k = 0; k < 25; ++k) gu[2][k] = t[k];
  } else if (d->src_type == AXG_DIPOLE) {
    f_over_s_el(s, axis, &w, u2, t);
    for (int k = 0; k < 25; ++k) gu[2][k] = 2 * t[k];
    for (int k = 0; k < 25; ++k) tmp[k] = u1[k] - u2[k];
    grad_el(s, axis, &w, tmp, b1s, b1z);
    f_over_s_el(s, axis, &w, u3, t);
    for (int k = 0; k < 25; ++k) {
      gu[4][k] = -t[k] - b1z[k];
      gu[6][k] = -gu[2][k] - b1s[k];
    }
  } else {
    for (int k = 0; k < 25; ++k) tmp[k] = u1[k] - 2 * u2[k];
    f_over_s_el(s, axis, &w, tmp, t);
    for (int k = 0; k < 25; ++k) gu[2][k] = t[k];
    grad_el(s, axis, &w, u2, b1s, b1z);
    f_over_s_el(s, axis, &w, u3, t);
    for (int k = 0; k < 25; ++k) tmp[k] = u2[k] - 2 * u1[k];
    f_over_s_el(s, axis, &w, tmp, t2);
    for (int k = 0; k < 25; ++k) {
      gu[4][k] = -2 * t[k] - b1z[k];
      gu[6][k] = t2[k] - b1s[k];
    }
  }
}

/* time_step_memvars_4, SOLVER/attenuation.f90:210-334.
 * memvar(0:4,0:4,6,n_sls,nel), src_tr_tm1(0:4,0:4,nel), src_dev_tm1(0:4,0:4,6,nel). */
void ORC(time_step_memvars_4)(const axg_mesh_desc *d, REAL *memvar, const REAL *disp, REAL *src_tr_tm1_glob,
                              REAL *src_dev_tm1_glob) {
  spec s;
  load_spec(d, &s);
  const int64_t ne = d->nel_solid, cs = 25 * ne;
  const int nsls = d->n_sls;
  const double third = 1.0 / 3.0;
  unsigned char *ax = axis_flags(d->nel_solid, d->naxel_solid, d->ax_el_solid);
#pragma omp parallel
  {
  double a_mu[32], a_ka[32];
  double Qmu_last = NAN, Qka_last = NAN;
#pragma omp for schedule(static)
  for (int64_t e = 0; e < ne; ++e) {
    REAL gu[7][25];
    strain_att_4(d, &s, e, ax[e], disp + 25 * e, disp + cs + 25 * e, disp + 2 * cs + 25 * e, gu);
    if (!((double)d->Q_mu[e] == Qmu_last)) {
      Qmu_last = d->Q_mu[e];
      ORC(sls_weights)(d, Qmu_last, a_mu);
    }
    if (!((double)d->Q_kappa[e] == Qka_last)) {
      Qka_last = d->Q_kappa[e];
      ORC(sls_weights)(d, Qka_last, a_ka);
    }
    REAL tr[25], src_tr[25], src_dev[7][25];
    for (int k = 0; k < 25; ++k) tr[k] = gu[1][k] + gu[2][k] + gu[3][k];
    const float *dmu = d->delta_mu + 25 * e, *dka = d->delta_kappa + 25 * e;
    for (int c = 1; c <= 6; ++c)
      for (int k = 0; k < 25; ++k) src_dev[c][k] = 0;
    for (int k = 0; k < 25; ++k) {
      const REAL dm = (REAL)dmu[k];
      src_tr[k] = (REAL)dka[k] * tr[k];
      for (int c = 1; c <= 3; ++c)
        src_dev[c][k] = (REAL)((double)(dm * 2) * ((double)gu[c][k] - (double)tr[k] * third));
      src_dev[5][k] = dm * gu[5][k];
      if (d->src_type != AXG_MONOPOLE) {
        src_dev[4][k] = dm * gu[4][k];
        src_dev[6][k] = dm * gu[6][k];
      }
    }
    REAL *trm1 = src_tr_tm1_glob + 25 * e, *devm1 = src_dev_tm1_glob + 150 * e;
    for (int j = 0; j < nsls; ++j) {
      const double ft = d->ts_fac_t[j], ftm1 = d->ts_fac_tm1[j], ex = d->exp_w_j_deltat[j];
      REAL *R = memvar + 25 * 6 * (j + (int64_t)nsls * e);
      for (int k = 0; k < 25; ++k) {
        const REAL trb = (REAL)(ft * a_ka[j] * src_tr[k] + ftm1 * a_ka[j] * trm1[k]);
        REAL db[7];
        for (int c = 1; c <= 6; ++c)
          db[c] = (REAL)(ft * a_mu[j] * src_dev[c][k] + ftm1 * a_mu[j] * devm1[k + 25 * (c - 1)]);
        R[k + 25 * 0] = (REAL)(ex * R[k + 25 * 0] + db[1] + trb);
        R[k + 25 * 1] = (REAL)(ex * R[k + 25 * 1] + db[2] + trb);
        R[k + 25 * 2] = (REAL)(ex * R[k + 25 * 2] + db[3] + trb);
        R[k + 25 * 4] = (REAL)(ex * R[k + 25 * 4] + db[5]);
        if (d->src_type != AXG_MONOPOLE) {
          R[k + 25 * 3] = (REAL)(ex * R[k + 25 * 3] + db[4]);
          R[k + 25 * 5] = (REAL)(ex * R[k + 25 * 5] + db[6]);
        }
      }
    }
    for (int k = 0; k < 25; ++k) {
      trm1[k] = src_tr[k];
      for (int c = 1; c <= 6; ++c) devm1[k + 25 * (c - 1)] = src_dev[c][k];
    }
  }
  }
  free(ax);
}

/* glob_anel_stiffness_{mono,di,quad}_4 (SOLVER/stiffness_mono.f90:409-507,
 * SOLVER/stiffness_di.f90:604-723, SOLVER/stiffness_quad.f90:555-669):
 * subtracts the divergence of the summed memory-variable stress.  The
 * dipole's axial z term adds outerprod(G0, V2) as the reference writes it. */
void ORC(anel_stiffness_4)(const axg_mesh_desc *d, const REAL *R, REAL *gs) {
  spec s;
  load_spec(d, &s);
  const int64_t ne = d->nel_solid, cs = 25 * ne;
  const int nsls = d->n_sls;
  unsigned char *ax = axis_flags(d->nel_solid, d->naxel_solid, d->ax_el_solid);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < ne; ++e) {
    mat5 yl, vse, vsx, vze, vzx, r[7];
    load_mat(yl, d->Y + 25 * e);
    load_mat(vse, d->V_s_eta + 25 * e);
    load_mat(vsx, d->V_s_xi + 25 * e);
    load_mat(vze, d->V_z_eta + 25 * e);
    load_mat(vzx, d->V_z_xi + 25 * e);
    for (int c = 1; c <= 6; ++c)
      for (int k = 0; k < 25; ++k) r[c][k] = 0;
    for (int j = 0; j < nsls; ++j)
      for (int c = 1; c <= 6; ++c)
        for (int k = 0; k < 25; ++k) r[c][k] = r[c][k] + R[k + 25 * ((c - 1) + 6 * (j + (int64_t)nsls * e))];
    const REAL *G = ax[e] ? s.G1 : s.G2;
    vec5 y0l = {0}, v0se = {0}, v0sx = {0}, v0ze = {0}, v0zx = {0}, V1, V2, V3;
    if (ax[e]) {
      for (int k = 0; k < 5; ++k) {
        y0l[k] = (REAL)d->Y0[5 * e + k];
        v0se[k] = (REAL)d->V0_s_eta[5 * e + k];
        v0sx[k] = (REAL)d->V0_s_xi[5 * e + k];
        v0ze[k] = (REAL)d->V0_z_eta[5 * e + k];
        v0zx[k] = (REAL)d->V0_z_xi[5 * e + k];
      }
    }
    mat5 S1a, S2a, S1b, S2b, S1z, S2z, X1, X2, X3, X4, X5, X6, la, lb, lz, op;
    REAL *g1 = gs + 25 * e, *g2 = g1 + cs, *g3 = g2 + cs;
    if (d->src_type == AXG_MONOPOLE) {
      for (int k = 0; k < 25; ++k) {
        S1a[k] = vze[k] * r[1][k] + vse[k] * r[5][k];
        S2a[k] = vzx[k] * r[1][k] + vsx[k] * r[5][k];
        S1z[k] = vze[k] * r[5][k] + vse[k] * r[3][k];
        S2z[k] = vzx[k] * r[5][k] + vsx[k] * r[3][k];
      }
      mxm_4(G, S1a, X1);
      mxm_4(G, S1z, X3);
      mxm_4(S2a, s.G2T, X2);
      mxm_4(S2z, s.G2T, X4);
      for (int k = 0; k < 25; ++k) {
        la[k] = X1[k] + X2[k] + yl[k] * r[2][k];
        lz[k] = X3[k] + X4[k];
      }
      if (ax[e]) {
        for (int j = 0; j < 5; ++j) {
          V1[j] = v0ze[j] * A(r[1], 0, j) + v0se[j] * A(r[5], 0, j) + y0l[j] * A(r[2], 0, j);
          V2[j] = v0ze[j] * A(r[5], 0, j) + v0se[j] * A(r[3], 0, j);
          V3[j] = v0zx[j] * A(r[5], 0, j) + v0sx[j] * A(r[3], 0, j);
        }
        outerprod_4(s.G0, V1, op);
        for (int k = 0; k < 25; ++k) la[k] = la[k] + op[k];
        vec5 V4;
        vxm_4(V3, s.G2T, V4);
        outerprod_4(s.G0, V2, op);
        for (int k = 0; k < 25; ++k) lz[k] = lz[k] + op[k];
        for (int j = 0; j < 5; ++j) A(lz, 0, j) = A(lz, 0, j) + V4[j];
      }
      for (int k = 0; k < 25; ++k) {
        g1[k] = g1[k] - la[k];
        g3[k] = g3[k] - lz[k];
      }
    } else if (d->src_type == AXG_DIPOLE) {
      mat5 r16m, r54m, r16p, r54p;
      for (int k = 0; k < 25; ++k) {
        r16m[k] = r[1][k] - r[6][k];
        r54m[k] = r[5][k] - r[4][k];
        r16p[k] = r[1][k] + r[6][k];
        r54p[k] = r[5][k] + r[4][k];
        S1a[k] = vze[k] * r16m[k] + vse[k] * r54m[k];
        S2a[k] = vzx[k] * r16m[k] + vsx[k] * r54m[k];
        S1b[k] = vze[k] * r16p[k] + vse[k] * r54p[k];
        S2b[k] = vzx[k] * r16p[k] + vsx[k] * r54p[k];
        S1z[k] = vze[k] * r[5][k] + vse[k] * r[3][k];
        S2z[k] = vzx[k] * r[5][k] + vsx[k] * r[3][k];
      }
      mxm_4(G, S1a, X1);
      mxm_4(G, S1b, X3);
      mxm_4(G, S1z, X5);
      mxm_4(S2a, s.G2T, X2);
      mxm_4(S2b, s.G2T, X4);
      mxm_4(S2z, s.G2T, X6);
      for (int k = 0; k < 25; ++k) {
        la[k] = X1[k] + X2[k];
        lb[k] = X3[k] + X4[k] + 2 * yl[k] * (r[2][k] - r[6][k]);
        lz[k] = X5[k] + X6[k] - yl[k] * r[4][k];
      }
      if (ax[e]) {
        for (int j = 0; j < 5; ++j) {
          V1[j] = v0ze[j] * (A(r[1], 0, j) - A(r[6], 0, j)) + v0se[j] * (A(r[5], 0, j) - A(r[4], 0, j));
          V2[j] = v0zx[j] * (A(r[1], 0, j) - A(r[6], 0, j)) + v0sx[j] * (A(r[5], 0, j) - A(r[4], 0, j));
        }
        vxm_4(V2, s.G2T, V3);
        outerprod_4(s.G0, V1, op);
        for (int k = 0; k < 25; ++k) la[k] = la[k] + op[k];
        for (int j = 0; j < 5; ++j) A(la, 0, j) = A(la, 0, j) + V3[j];
        for (int j = 0; j < 5; ++j)
          V1[j] = v0ze[j] * (A(r[1], 0, j) + A(r[6], 0, j)) + v0se[j] * (A(r[5], 0, j) + A(r[4], 0, j)) +
                  y0l[j] * 2 * (A(r[2], 0, j) - A(r[6], 0, j));
        outerprod_4(s.G0, V1, op);
        for (int k = 0; k < 25; ++k) lb[k] = lb[k] + op[k];
        outerprod_4(s.G0, V2, op);  /* (V1 of the z component is formed but not used) */
        for (int k = 0; k < 25; ++k) lz[k] = lz[k] + op[k];
      }
      for (int k = 0; k < 25; ++k) {
        g1[k] = g1[k] - la[k];
        g2[k] = g2[k] - lb[k];
        g3[k] = g3[k] - lz[k];
      }
    } else {
      for (int k = 0; k < 25; ++k) {
        S1a[k] = vze[k] * r[1][k] + vse[k] * r[5][k];
        S2a[k] = vzx[k] * r[1][k] + vsx[k] * r[5][k];
        S1b[k] = vze[k] * r[6][k] + vse[k] * r[4][k];
        S2b[k] = vzx[k] * r[6][k] + vsx[k] * r[4][k];
        S1z[k] = vze[k] * r[5][k] + vse[k] * r[3][k];
        S2z[k] = vzx[k] * r[5][k] + vsx[k] * r[3][k];
      }
      mxm_4(G, S1a, X1);
      mxm_4(G, S1b, X3);
      mxm_4(G, S1z, X5);
      mxm_4(S2a, s.G2T, X2);
      mxm_4(S2b, s.G2T, X4);
      mxm_4(S2z, s.G2T, X6);
      for (int k = 0; k < 25; ++k) {
        la[k] = X1[k] + X2[k] + yl[k] * (r[2][k] - 2 * r[6][k]);
        lb[k] = -X3[k] - X4[k] + yl[k] * (r[6][k] - 2 * r[2][k]);
        lz[k] = X5[k] + X6[k] - 2 * yl[k] * r[4][k];
      }
      if (ax[e]) {
        for (int j = 0; j < 5; ++j) V1[j] = v0ze[j] * A(r[1], 0, j) + y0l[j] * (A(r[2], 0, j) - 2 * A(r[6], 0, j));
        outerprod_4(s.G0, V1, op);
        for (int k = 0; k < 25; ++k) la[k] = la[k] + op[k];
        for (int j = 0; j < 5; ++j) V1[j] = -v0ze[j] * A(r[6], 0, j) + y0l[j] * (A(r[6], 0, j) - 2 * A(r[2], 0, j));
        outerprod_4(s.G0, V1, op);
        for (int k = 0; k < 25; ++k) lb[k] = lb[k] + op[k];
        for (int j = 0; j < 5; ++j) V1[j] = v0se[j] * A(r[3], 0, j);
        outerprod_4(s.G0, V1, op);
        for (int k = 0; k < 25; ++k) lz[k] = lz[k] + op[k];
      }
      for (int k = 0; k < 25; ++k) {
        g1[k] = g1[k] - la[k];
        g2[k] = g2[k] - lb[k];
        g3[k] = g3[k] - lz[k];
      }
    }
  }
  free(ax);
}

/* the attenuation variant the descriptor selects */
static void anel_stiffness(const axg_mesh_desc *d, const REAL *R, REAL *gs) {
  if (d->att_coarse_grained) ORC(anel_stiffness_cg4)(d, R, gs);
  else ORC(anel_stiffness_4)(d, R, gs);
}
static void time_step_memvars(const axg_mesh_desc *d, REAL *memvar, const REAL *disp, REAL *trm1, REAL *devm1) {
  if (d->att_coarse_grained) ORC(time_step_memvars_cg4)(d, memvar, disp, trm1, devm1);
  else ORC(time_step_memvars_4)(d, memvar, disp, trm1, devm1);
}

/* ------------------------------------------------------------ assembly */

/* the edge-point walk of pdistsum_*: ipol fastest, interior points skipped */
static int edge_points(int *ipt_off) {
  int n = 0;
  for (int j = 0; j < 5; ++j)
    for (int i = 0; i < 5; ++i)
      if (j == 0 || j == 4 || i == 0 || i == 4) ipt_off[n++] = i + 5 * j;
  return n;
}

/* pdistsum_solid (serial), SOLVER/commun.F90:69-171 */
void ORC(pdistsum_solid)(const axg_mesh_desc *d, REAL *vec, int nc) {
  const int64_t ne = d->nel_solid, cs = 25 * ne, ng = d->nglob_solid;
  REAL *g = (REAL *)calloc((size_t)(ng * nc > 0 ? ng * nc : 1), sizeof(REAL));
  int ep[16];
  const int nep = edge_points(ep);
  for (int64_t e = 0; e < ne; ++e)
    for (int q = 0; q < nep; ++q) {
      const int64_t p = 25 * e + ep[q], idest = d->igloc_solid[p] - 1;
      for (int c = 0; c < nc; ++c) g[idest + ng * c] = g[idest + ng * c] + vec[p + cs * c];
    }
  for (int64_t e = 0; e < ne; ++e)
    for (int q = 0; q < nep; ++q) {
      const int64_t p = 25 * e + ep[q], idest = d->igloc_solid[p] - 1;
      for (int c = 0; c < nc; ++c) vec[p + cs * c] = g[idest + ng * c];
    }
  free(g);
}

/* pdistsum_fluid (serial), SOLVER/commun.F90:180-283 */
void ORC(pdistsum_fluid)(const axg_mesh_desc *d, REAL *vec) {
  const int64_t ne = d->nel_fluid, ng = d->nglob_fluid;
  REAL *g = (REAL *)calloc((size_t)(ng > 0 ? ng : 1), sizeof(REAL));
  int ep[16];
  const int nep = edge_points(ep);
  for (int64_t e = 0; e < ne; ++e)
    for (int q = 0; q < nep; ++q) {
      const int64_t p = 25 * e + ep[q];
      g[d->igloc_fluid[p] - 1] = g[d->igloc_fluid[p] - 1] + vec[p];
    }
  for (int64_t e = 0; e < ne; ++e)
    for (int q = 0; q < nep; ++q) {
      const int64_t p = 25 * e + ep[q];
      vec[p] = g[d->igloc_fluid[p] - 1];
    }
  free(g);
}

/* ------------------------------------------------------------ masks, coupling */

/* apply_axis_mask_{onecomp,twocomp,threecomp} as selected by the pole type */
static void mask_solid(const axg_mesh_desc *d, REAL *u) {
  const int64_t cs = 25 * (int64_t)d->nel_solid;
  const int c0 = d->src_type == AXG_MONOPOLE ? 0 : (d->src_type == AXG_DIPOLE ? 1 : 0);
  const int c1 = d->src_type == AXG_MONOPOLE ? 0 : 2;
  for (int k = 0; k < d->naxel_solid; ++k) {
    const int64_t e = d->ax_el_solid[k] - 1;
    for (int c = c0; c <= c1; ++c)
      for (int j = 0; j < 5; ++j) u[25 * e + 5 * j + cs * c] = 0;
  }
}

/* apply_axis_mask_scal */
static void mask_fluid(const axg_mesh_desc *d, REAL *chi) {
  for (int k = 0; k < d->naxel_fluid; ++k) {
    const int64_t e = d->ax_el_fluid[k] - 1;
    for (int j = 0; j < 5; ++j) chi[25 * e + 5 * j] = 0;
  }
}

/* bdry_copy2fluid, SOLVER/time_evol_wave.F90:1532-1571 */
static void bdry_copy2fluid(const axg_mesh_desc *d, REAL *uflu, const REAL *usol) {
  const int64_t cs = 25 * (int64_t)d->nel_solid, nb = d->nel_bdry;
  for (int64_t b = 0; b < nb; ++b) {
    const int js = d->bdry_jpol_solid[b], jf = d->bdry_jpol_fluid[b];
    const int64_t es = d->bdry_solid_el[b] - 1, ef = d->bdry_fluid_el[b] - 1;
    for (int i = 0; i < 5; ++i) {
      const REAL b1 = (REAL)d->bdry_matr[i + 5 * b], b2 = (REAL)d->bdry_matr[i + 5 * (b + nb)];
      const int64_t ps = 25 * es + i + 5 * js, pf = 25 * ef + i + 5 * jf;
      if (d->src_type == AXG_DIPOLE)
        uflu[pf] = uflu[pf] - b1 * (usol[ps] + usol[ps + cs]) - b2 * usol[ps + 2 * cs];
      else
        uflu[pf] = uflu[pf] - b1 * usol[ps] - b2 * usol[ps + 2 * cs];
    }
  }
}

/* bdry_copy2solid, SOLVER/time_evol_wave.F90:1577-1611 */
static void bdry_copy2solid(const axg_mesh_desc *d, REAL *usol, const REAL *uflu) {
  const int64_t cs = 25 * (int64_t)d->nel_solid, nb = d->nel_bdry;
  for (int64_t b = 0; b < nb; ++b) {
    const int js = d->bdry_jpol_solid[b], jf = d->bdry_jpol_fluid[b];
    const int64_t es = d->bdry_solid_el[b] - 1, ef = d->bdry_fluid_el[b] - 1;
    for (int i = 0; i < 5; ++i) {
      const REAL b1 = (REAL)d->bdry_matr[i + 5 * b], b2 = (REAL)d->bdry_matr[i + 5 * (b + nb)];
      const int64_t ps = 25 * es + i + 5 * js, pf = 25 * ef + i + 5 * jf;
      usol[ps] = usol[ps] + b1 * uflu[pf];
      if (d->src_type == AXG_DIPOLE) usol[ps + cs] = usol[ps + cs] + b1 * uflu[pf];
      usol[ps + 2 * cs] = usol[ps + 2 * cs] + b2 * uflu[pf];
    }
  }
}

/* ------------------------------------------------ stiffness + assembly (cfg 2) */

/* u_gvec(nglob,3) -> f_gvec(nglob,3):
 * scatter to element-local, axis mask (in place, as before the stiffness
 * call), glob_stiffness, axis mask of the result, pdistsum_solid, gather. */
void ORC(stiffness_assembled)(const axg_mesh_desc *d, const REAL *u_g, REAL *f_g) {
  const int64_t ne = d->nel_solid, cs = 25 * ne, ng = d->nglob_solid;
  REAL *u = (REAL *)malloc(sizeof(REAL) * (size_t)(3 * cs > 0 ? 3 * cs : 1));
  REAL *f = (REAL *)malloc(sizeof(REAL) * (size_t)(3 * cs > 0 ? 3 * cs : 1));
  for (int64_t p = 0; p < cs; ++p)
    for (int c = 0; c < 3; ++c) u[p + cs * c] = u_g[d->igloc_solid[p] - 1 + ng * c];
  mask_solid(d, u);
  ORC(stiffness_solid)(d, u, f);
  mask_solid(d, f);
  ORC(pdistsum_solid)(d, f, 3);
  for (int64_t p = 0; p < cs; ++p)
    for (int c = 0; c < 3; ++c) f_g[d->igloc_solid[p] - 1 + ng * c] = f[p + cs * c];
  free(u);
  free(f);
}

/* ------------------------------------------------------------ time loop */

typedef struct ORC(state) {
  REAL *disp, *velo, *acc0, *acc1;   /* (0:4,0:4,nel_solid,3) */
  REAL *chi, *dchi, *ddchi0, *ddchi1; /* (0:4,0:4,nel_fluid) */
  REAL *memvar;                       /* (1:4,6,n_sls,nel_solid) */
  REAL *src_tr_tm1, *src_dev_tm1;     /* (1:4,nel), (1:4,6,nel) */
} ORC(state);

/* Runs sf_time_loop_newmark for iterations first_iter..first_iter+n_iter-1 on
 * the given state (zeroed by the caller for a fresh run), sampling receivers
 * into rec(nseismo_cap,3,num_rec) at iseismo (0-based, advanced in place).
 * Returns 0, or AXG_ERR_BLOWUP with *blowup_iter set. */
int ORC(time_loop)(const axg_mesh_desc *d, REAL *disp, REAL *velo, REAL *acc0, REAL *chi,
                   REAL *dchi, REAL *ddchi0, REAL *memvar, REAL *src_tr_tm1, REAL *src_dev_tm1,
                   int32_t first_iter, int32_t n_iter, float *rec, int32_t nseismo_cap,
                   int32_t *iseismo, int32_t *blowup_iter) {
  const int64_t nes = d->nel_solid, cs = 25 * nes, nef = d->nel_fluid, cf = 25 * nef;
  const double deltat = d->deltat, half_dt = 0.5 * deltat, half_dt_sq = 0.5 * deltat * deltat;
  const int mono = d->src_type == AXG_MONOPOLE;
  REAL *acc1 = (REAL *)calloc((size_t)(3 * cs > 0 ? 3 * cs : 1), sizeof(REAL));
  REAL *ddchi1 = (REAL *)calloc((size_t)(cf > 0 ? cf : 1), sizeof(REAL));
  const double thresh = 10.0 * fabs(d->magnitude);
  int status = 0;

  for (int32_t iter = first_iter; iter < first_iter + n_iter; ++iter) {
    /* runtime_info blow-up guard on disp(1,1,:,:) */
    REAL mx = 0;
    for (int64_t e = 0; e < nes; ++e)
      for (int c = 0; c < 3; ++c) {
        REAL v = (REAL)fabs((double)disp[25 * e + 1 + 5 * 1 + cs * c]);
        if (v > mx) mx = v;
      }
    if ((double)mx > thresh) {
      if (blowup_iter) *blowup_iter = iter;
      status = AXG_ERR_BLOWUP;
      break;
    }
    /* predictor */
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < cf; ++p)
      chi[p] = (REAL)((double)chi[p] + deltat * dchi[p] + half_dt_sq * ddchi0[p]);
    for (int c = 0; c < 3; ++c) {
      if (c == 1 && mono) continue;
#pragma omp parallel for schedule(static)
      for (int64_t p = 0; p < cs; ++p)
        disp[p + cs * c] =
            (REAL)((double)disp[p + cs * c] + deltat * velo[p + cs * c] + half_dt_sq * acc0[p + cs * c]);
    }
    if (!mono) mask_fluid(d, chi);
    /* fluid */
    if (nef > 0) {
      ORC(stiffness_fluid)(d, chi, ddchi1);
      if (d->fluid_src && d->stf[iter - 1] != 0) {
        const REAL stf1 = (REAL)d->stf[iter - 1];
        for (int k = 0; k < d->nelsrc; ++k) {
          const int64_t e = d->ielsrc[k] - 1;
          for (int q = 0; q < 25; ++q)
            ddchi1[25 * e + q] = ddchi1[25 * e + q] - (REAL)d->source_term_fl[q + 25 * k] * stf1;
        }
      }
      bdry_copy2fluid(d, ddchi1, disp);
      if (!mono) mask_fluid(d, ddchi1);
      if (d->fluid_free_surface_mask)
        for (int64_t p = 0; p < cf; ++p) ddchi1[p] = ddchi1[p] * (REAL)d->fluid_free_surface_mask[p];
      ORC(pdistsum_fluid)(d, ddchi1);
    }
    /* solid */
    mask_solid(d, disp);
    ORC(stiffness_solid)(d, disp, acc1);
    if (d->anel_true) anel_stiffness(d, memvar, acc1);
    if (nef > 0) {
      for (int64_t p = 0; p < cf; ++p) ddchi1[p] = -(REAL)d->inv_mass_fluid[p] * ddchi1[p];
      if (d->have_absorbing_bc)
        for (int64_t p = 0; p < cf; ++p) {
          const REAL g = (REAL)d->fluid_absorbing_gamma[p];
          ddchi1[p] = ddchi1[p] - 2 * g * dchi[p] - g * g * chi[p];
        }
      bdry_copy2solid(d, acc1, ddchi1);
    }
    mask_solid(d, acc1);
    ORC(pdistsum_solid)(d, acc1, 3);
    if (d->anel_true) time_step_memvars(d, memvar, disp, src_tr_tm1, src_dev_tm1);
    for (int64_t p = 0; p < cf; ++p) {
      dchi[p] = (REAL)((double)dchi[p] + half_dt * (ddchi0[p] + ddchi1[p]));
      ddchi0[p] = ddchi1[p];
    }
    if (!d->fluid_src && d->stf[iter - 1] != 0) {
      const REAL stf1 = (REAL)d->stf[iter - 1];
      for (int k = 0; k < d->nelsrc; ++k) {
        const int64_t e = d->ielsrc[k] - 1;
        for (int c = 0; c < 3; ++c)
          for (int q = 0; q < 25; ++q)
            acc1[25 * e + q + cs * c] =
                acc1[25 * e + q + cs * c] - (REAL)d->source_term_el[q + 25 * k + 200 * c] * stf1;
      }
    }
    /* corrector: component order 1, 3, 2 as in the reference */
    const int order[3] = {0, 2, 1};
    for (int oc = 0; oc < 3; ++oc) {
      const int c = order[oc];
      if (c == 1 && mono) continue;
#pragma omp parallel for schedule(static)
      for (int64_t p = 0; p < cs; ++p) {
        const int64_t q = p + cs * c;
        const REAL im = (REAL)d->inv_mass_rho[p];
        REAL a;
        if (c == 2 && d->src_type == AXG_DIPOLE)
          a = (REAL)(-2.0 * (double)im * (double)acc1[q]);
        else
          a = -im * acc1[q];
        if (d->have_absorbing_bc) {
          const REAL g = (REAL)d->solid_absorbing_gamma[p];
          a = a - 2 * g * velo[q] - g * g * disp[q];
        }
        acc1[q] = a;
        velo[q] = (REAL)((double)velo[q] + half_dt * (acc0[q] + acc1[q]));
        acc0[q] = acc1[q];
      }
    }
    /* dump_stuff: seismograms every seis_it steps */
    if (d->num_rec > 0 && rec && d->seis_it > 0 && iter % d->seis_it == 0) {
      if (*iseismo < nseismo_cap) {
        const int64_t n = nseismo_cap, is = *iseismo;
        for (int r = 0; r < d->num_rec; ++r) {
          const int64_t e = d->recfile_el[r] - 1;
          const int ip = d->recfile_el[r + d->num_rec], jp = d->recfile_el[r + 2 * d->num_rec];
          const int64_t p = 25 * e + ip + 5 * jp;
          REAL v1, v2, v3;
          if (d->src_type == AXG_MONOPOLE) {
            v1 = disp[p]; v2 = 0; v3 = disp[p + 2 * cs];
          } else if (d->src_type == AXG_DIPOLE) {
            v1 = disp[p] + disp[p + cs]; v2 = disp[p] - disp[p + cs]; v3 = disp[p + 2 * cs];
          } else {
            v1 = disp[p]; v2 = disp[p + cs]; v3 = disp[p + 2 * cs];
          }
          rec[is + n * (0 + 3 * (int64_t)r)] = (float)v1;
          rec[is + n * (1 + 3 * (int64_t)r)] = (float)v2;
          rec[is + n * (2 + 3 * (int64_t)r)] = (float)v3;
        }
      }
      *iseismo += 1;
    }
  }
  free(acc1);
  free(ddchi1);
  return status;
}

/* symplectic_time_loop (SOLVER/time_evol_wave.F90:516-742): iterations
 * first_iter..first_iter+n_iter-1 of an nstages scheme whose drifts
 * coefd(1:nstages+1) and kicks coefv(1:nstages) are given times deltat;
 * stf_stages(niter, nstages) holds the source time function at the stage
 * times.  disp, velo (0:4,0:4,nel_solid,3), chi, dchi (0:4,0:4,nel_fluid)
 * carry the state; with attenuation every stage adds the anelastic stiffness
 * of the previous step's memory variables, which time_step_memvars updates
 * after the final drift (memvar, src_*_tm1 as in time_loop); seismograms as
 * in time_loop. */
int ORC(time_loop_symplectic)(const axg_mesh_desc *d, int32_t nstages, const double *coefd, const double *coefv,
                              const float *stf_stages, REAL *disp, REAL *velo, REAL *chi, REAL *dchi,
                              REAL *memvar, REAL *src_tr_tm1, REAL *src_dev_tm1,
                              int32_t first_iter, int32_t n_iter, float *rec, int32_t nseismo_cap,
                              int32_t *iseismo, int32_t *blowup_iter) {
  const int64_t nes = d->nel_solid, cs = 25 * nes, nef = d->nel_fluid, cf = 25 * nef;
  const int mono = d->src_type == AXG_MONOPOLE, di = d->src_type == AXG_DIPOLE;
  REAL *acc = (REAL *)calloc((size_t)(3 * cs > 0 ? 3 * cs : 1), sizeof(REAL));
  REAL *ddchi = (REAL *)calloc((size_t)(cf > 0 ? cf : 1), sizeof(REAL));
  const double thresh = 10.0 * fabs(d->magnitude);
  int status = 0;
  for (int32_t iter = first_iter; iter < first_iter + n_iter; ++iter) {
    REAL mx = 0;
    for (int64_t e = 0; e < nes; ++e)
      for (int c = 0; c < 3; ++c) {
        REAL v = (REAL)fabs((double)disp[25 * e + 1 + 5 * 1 + cs * c]);
        if (v > mx) mx = v;
      }
    if ((double)mx > thresh) {
      if (blowup_iter) *blowup_iter = iter;
      status = AXG_ERR_BLOWUP;
      break;
    }
    for (int i = 0; i < nstages; ++i) {
      for (int64_t p = 0; p < cf; ++p) chi[p] = (REAL)((double)chi[p] + (double)dchi[p] * coefd[i]);
      for (int c = 0; c < 3; ++c) {
        if (c == 1 && mono) continue;
        for (int64_t p = 0; p < cs; ++p)
          disp[p + cs * c] = (REAL)((double)disp[p + cs * c] + (double)velo[p + cs * c] * coefd[i]);
      }
      if (nef > 0) {
        if (!mono) mask_fluid(d, chi);
        ORC(stiffness_fluid)(d, chi, ddchi);
        bdry_copy2fluid(d, ddchi, disp);
        if (!mono) mask_fluid(d, ddchi);
        ORC(pdistsum_fluid)(d, ddchi);
      }
      mask_solid(d, disp);
      ORC(stiffness_solid)(d, disp, acc);
      /* glob_anel_stiffness_*: the memory variables of the previous step */
      if (d->anel_true) anel_stiffness(d, memvar, acc);
      if (nef > 0) {
        for (int64_t p = 0; p < cf; ++p) ddchi[p] = -ddchi[p] * (REAL)d->inv_mass_fluid[p];
        if (d->have_absorbing_bc)
          for (int64_t p = 0; p < cf; ++p) {
            const REAL g = (REAL)d->fluid_absorbing_gamma[p];
            ddchi[p] = ddchi[p] - 2 * g * dchi[p] - g * g * chi[p];
          }
        bdry_copy2solid(d, acc, ddchi);
      }
      mask_solid(d, acc);
      ORC(pdistsum_solid)(d, acc, 3);
      for (int64_t p = 0; p < cf; ++p) dchi[p] = (REAL)((double)dchi[p] + coefv[i] * (double)ddchi[p]);
      const REAL stf1 = (REAL)stf_stages[(int64_t)(iter - 1) + (int64_t)d->niter * i];
      if (stf1 != 0)
        for (int k = 0; k < d->nelsrc; ++k) {
          const int64_t e = d->ielsrc[k] - 1;
          for (int c = 0; c < 3; ++c)
            for (int q = 0; q < 25; ++q)
              acc[25 * e + q + cs * c] = acc[25 * e + q + cs * c] - (REAL)d->source_term_el[q + 25 * k + 200 * c] * stf1;
        }
      const int order[3] = {0, 1, 2};
      for (int oc = 0; oc < 3; ++oc) {
        const int c = order[oc];
        if (c == 1 && mono) continue;
        for (int64_t p = 0; p < cs; ++p) {
          const int64_t q = p + cs * c;
          REAL a = -(REAL)d->inv_mass_rho[p] * acc[q];
          if (d->have_absorbing_bc) {
            const REAL g = (REAL)d->solid_absorbing_gamma[p];
            a = a - 2 * g * velo[q] - g * g * disp[q];
          }
          acc[q] = a;
          if (c == 2 && di)
            velo[q] = (REAL)((double)velo[q] + 2.0 * (double)acc[q] * coefv[i]);
          else
            velo[q] = (REAL)((double)velo[q] + (double)acc[q] * coefv[i]);
        }
      }
    }
    for (int64_t p = 0; p < cf; ++p) chi[p] = (REAL)((double)chi[p] + (double)dchi[p] * coefd[nstages]);
    for (int c = 0; c < 3; ++c) {
      if (c == 1 && mono) continue;
      for (int64_t p = 0; p < cs; ++p)
        disp[p + cs * c] = (REAL)((double)disp[p + cs * c] + (double)velo[p + cs * c] * coefd[nstages]);
    }
    /* time_step_memvars from the drifted displacement (SOLVER/time_evol_wave.F90:727-731) */
    if (d->anel_true) time_step_memvars(d, memvar, disp, src_tr_tm1, src_dev_tm1);
    if (d->num_rec > 0 && rec && d->seis_it > 0 && iter % d->seis_it == 0) {
      if (*iseismo < nseismo_cap) {
        const int64_t n = nseismo_cap, is = *iseismo;
        for (int r = 0; r < d->num_rec; ++r) {
          const int64_t e = d->recfile_el[r] - 1;
          const int ip = d->recfile_el[r + d->num_rec], jp = d->recfile_el[r + 2 * d->num_rec];
          const int64_t p = 25 * e + ip + 5 * jp;
          REAL v1, v2, v3;
          if (mono) {
            v1 = disp[p]; v2 = 0; v3 = disp[p + 2 * cs];
          } else if (di) {
            v1 = disp[p] + disp[p + cs]; v2 = disp[p] - disp[p + cs]; v3 = disp[p + 2 * cs];
          } else {
            v1 = disp[p]; v2 = disp[p + cs]; v3 = disp[p + 2 * cs];
          }
          rec[is + n * (0 + 3 * (int64_t)r)] = (float)v1;
          rec[is + n * (1 + 3 * (int64_t)r)] = (float)v2;
          rec[is + n * (2 + 3 * (int64_t)r)] = (float)v3;
        }
      }
      *iseismo += 1;
    }
  }
  free(acc);
  free(ddchi);
  return status;
}

/* The analytic-field pointwise-derivative known-answer test of the reference
 * (test_pntwsdrvtvs_solid, SOLVER/def_precomp_terms.f90:308-367) restricted to
 * the cg4 points: f given element-local (0:4,0:4,nel), out grad(1:4,2,nel). */
void ORC(gradient_cg4_all)(const axg_mesh_desc *d, const REAL *f, REAL *out) {
  spec s;
  load_spec(d, &s);
  unsigned char *ax = axis_flags(d->nel_solid, d->naxel_solid, d->ax_el_solid);
  for (int64_t e = 0; e < d->nel_solid; ++e) {
    REAL g[2][4];
    gradient_cg4(d, &s, e, ax[e], f + 25 * e, g);
    for (int k = 0; k < 4; ++k) {
      out[k + 8 * e] = g[0][k];
      out[4 + k + 8 * e] = g[1][k];
    }
  }
  free(ax);
}


/* ------------------------------------------------- kernel wavefield dumps */

/* compute_strain for one element of the solid (SOLVER/time_evol_wave.F90:
 * 1286-1345) or, from the fluid displacement (usz_s, usz_z), of the fluid
 * (:1347-1408): dsus, dsuz, dpup, straintrace[, dsup, dzup] into o[0..5]. */
static void strain_el(const spec *s, int axis, const pw_el *w, int pole, int fluid, const REAL *u1, const REAL *u2,
                      const REAL *u3, REAL *o[6]) {
  mat5 us, g1, g2, h1, h2, n1, n2, buff, t, t2, p1, p2;
  for (int k = 0; k < 25; ++k) us[k] = (!fluid && pole == AXG_DIPOLE) ? u1[k] + u2[k] : u1[k];
  grad_el(s, axis, w, us, g1, g2);  /* 1: dsus, 2: dzus */
  for (int k = 0; k < 25; ++k) o[0][k] = g1[k];
  grad_el(s, axis, w, u3, h1, h2);  /* axisym_gradient_*_add: 1: dzus + dsuz, 2: dsus + dzuz */
  for (int k = 0; k < 25; ++k) {
    n1[k] = g2[k] + h1[k];
    n2[k] = g1[k] + h2[k];
    n1[k] = n1[k] / (REAL)2;
    o[1][k] = n1[k];
  }
  if (fluid) {
    f_over_s_el(s, axis, w, u1, buff);                         /* us / s */
    for (int k = 0; k < 25; ++k) {
      o[2][k] = buff[k];
      o[3][k] = buff[k] + n2[k];
    }
    if (pole == AXG_MONOPOLE) return;
    f_over_s_el(s, axis, w, u3, t);                            /* uz / s */
    for (int k = 0; k < 25; ++k) {
      o[4][k] = pole == AXG_DIPOLE ? (-buff[k]) / (REAL)2 : -buff[k];
      o[5][k] = pole == AXG_DIPOLE ? t[k] / (REAL)2 : -t[k];
    }
    return;
  }
  if (pole == AXG_MONOPOLE) {
    f_over_s_el(s, axis, w, u1, buff);
  } else if (pole == AXG_DIPOLE) {
    f_over_s_el(s, axis, w, u2, t);
    for (int k = 0; k < 25; ++k) buff[k] = (REAL)2 * t[k];
  } else {
    for (int k = 0; k < 25; ++k) t[k] = u1[k] - (REAL)2 * u2[k];
    f_over_s_el(s, axis, w, t, buff);
  }
  for (int k = 0; k < 25; ++k) {
    o[2][k] = buff[k];
    o[3][k] = buff[k] + n2[k];
  }
  if (pole == AXG_DIPOLE) {
    for (int k = 0; k < 25; ++k) t2[k] = u1[k] - u2[k];
    grad_el(s, axis, w, t2, p1, p2);                           /* dsup, dzup */
    f_over_s_el(s, axis, w, u2, t);
    for (int k = 0; k < 25; ++k) o[4][k] = -t[k] - p1[k] / (REAL)2;
    f_over_s_el(s, axis, w, u3, t);
    for (int k = 0; k < 25; ++k) o[5][k] = -(t[k] + p2[k]) / (REAL)2;
  } else if (pole == AXG_QUADPOLE) {
    grad_el(s, axis, w, u2, p1, p2);
    for (int k = 0; k < 25; ++k) t2[k] = u1[k] + u2[k] / (REAL)2;
    f_over_s_el(s, axis, w, t2, t);
    for (int k = 0; k < 25; ++k) o[4][k] = -t[k] - p1[k] / (REAL)2;
    f_over_s_el(s, axis, w, u3, t);
    for (int k = 0; k < 25; ++k) o[5][k] = -t[k] - p2[k] / (REAL)2;
  }
}

/* pack(f(ibeg:iend, jbeg:jend, e)) of one element into field `fld` */
static void put_el(const axg_dump_desc *dd, REAL *out, int64_t nel, int64_t e, int64_t fld, const REAL *f) {
  const int ni = dd->iend - dd->ibeg + 1, nj = dd->jend - dd->jbeg + 1;
  REAL *o = out + (fld * nel + e) * (int64_t)(ni * nj);
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i < ni; ++i) o[i + ni * j] = f[(dd->ibeg + i) + 5 * (dd->jbeg + j)];
}

/* a solid field of element e, zero where the source mask applies */
static void put_sol(const axg_dump_desc *dd, REAL *out, int64_t nel, int64_t e, int64_t fld, int masked,
                    const REAL *f) {
  mat5 z;
  if (masked) {
    for (int k = 0; k < 25; ++k) z[k] = 0;
    f = z;
  }
  put_el(dd, out, nel, e, fld, f);
}

/* One snapshot of dump_stuff's fields (the layout of axg_wavefield_dump_layout)
 * from the element-local state; returns the number of fields written. */
int ORC(wavefield_dump)(const axg_mesh_desc *d, const axg_dump_desc *dd, const REAL *disp, const REAL *velo,
                        const REAL *chi, const REAL *dchi, REAL *out) {
  spec s;
  load_spec(d, &s);
  const int pole = d->src_type, type = dd->dump_type;
  const int nonmono = pole != AXG_MONOPOLE;
  const int64_t nes = d->nel_solid, nef = d->nel_fluid;
  const int ns = type == AXG_DUMP_STRAIN_ONLY ? (nonmono ? 6 : 4)
                 : type == AXG_DUMP_FULLFIELDS ? (nonmono ? 6 : 4) + (nonmono ? 3 : 2)
                 : type == AXG_DUMP_DISPL_VELO ? 2 * (nonmono ? 3 : 2)
                                                : (nonmono ? 3 : 2);
  const int nf = nef <= 0 ? 0
                 : type == AXG_DUMP_STRAIN_ONLY ? (nonmono ? 6 : 4)
                 : type == AXG_DUMP_FULLFIELDS ? (nonmono ? 6 : 4) + (nonmono ? 3 : 2)
                 : type == AXG_DUMP_DISPL_VELO ? 2
                                                : (nonmono ? 3 : 2);
  const int np = (dd->iend - dd->ibeg + 1) * (dd->jend - dd->jbeg + 1);
  REAL *fout = out + (int64_t)ns * nes * np;
  unsigned char *axs = axis_flags((int)nes, d->naxel_solid, d->ax_el_solid);
  mat5 buf[6], v3[3];
  REAL *o[6] = {buf[0], buf[1], buf[2], buf[3], buf[4], buf[5]};
  for (int64_t e = 0; e < nes; ++e) {
    const int64_t off = 25 * e;
    const pw_el w = {dd->DsDeta_over_J_sol + off, dd->DzDeta_over_J_sol + off, dd->DsDxi_over_J_sol + off,
                     dd->DzDxi_over_J_sol + off, dd->inv_s_solid + off};
    /* src_dump_type = 'mask': eradicate_src_elem_values / _vec_values
     * (SOLVER/wavefields_io.f90:1123-1153) zero the solid fields of the
     * elements ielsrc (taken as solid elements, as the reference does) */
    int masked = 0;
    if (dd->src_dump_mask)
      for (int k = 0; k < d->nelsrc; ++k) masked |= d->ielsrc[k] - 1 == e;
    const REAL *u1 = disp + off, *u2 = disp + 25 * nes + off, *u3 = disp + 50 * nes + off;
    const REAL *vv1 = velo + off, *vv2 = velo + 25 * nes + off, *vv3 = velo + 50 * nes + off;
    int fld = 0;
    /* the s, phi, z components as dump_*_global write them (dipole: s, phi from +, -) */
    const REAL *vecs[2][3] = {{u1, u2, u3}, {vv1, vv2, vv3}};
    if (type == AXG_DUMP_STRAIN_ONLY || type == AXG_DUMP_FULLFIELDS) {
      strain_el(&s, axs[e], &w, pole, 0, u1, u2, u3, o);
      for (int q = 0; q < (nonmono ? 6 : 4); ++q) put_sol(dd, out, nes, e, fld++, masked, o[q]);
    }
    for (int which = 0; which < 2; ++which) {
      const int want = which == 0 ? (type == AXG_DUMP_DISPL_ONLY || type == AXG_DUMP_DISPL_VELO)
                                  : (type == AXG_DUMP_DISPL_VELO || type == AXG_DUMP_FULLFIELDS);
      if (!want) continue;
      const REAL **x = vecs[which];
      const int global = type != AXG_DUMP_DISPL_VELO;  /* dump_*_global transform the dipole */
      for (int k = 0; k < 25; ++k) {
        v3[0][k] = (global && pole == AXG_DIPOLE) ? x[0][k] + x[1][k] : x[0][k];
        v3[1][k] = (global && pole == AXG_DIPOLE) ? x[0][k] - x[1][k] : x[1][k];
        v3[2][k] = x[2][k];
      }
      put_sol(dd, out, nes, e, fld++, masked, v3[0]);
      if (nonmono) put_sol(dd, out, nes, e, fld++, masked, v3[1]);
      put_sol(dd, out, nes, e, fld++, masked, v3[2]);
    }
  }
  free(axs);
  if (nef > 0) {
    unsigned char *axf = axis_flags((int)nef, d->naxel_fluid, d->ax_el_fluid);
    mat5 c1, c2, zero;
    for (int k = 0; k < 25; ++k) zero[k] = 0;
    for (int64_t e = 0; e < nef; ++e) {
      const int64_t off = 25 * e;
      const pw_el w = {dd->DsDeta_over_J_flu + off, dd->DzDeta_over_J_flu + off, dd->DsDxi_over_J_flu + off,
                       dd->DzDxi_over_J_flu + off, dd->inv_s_fluid + off};
      const float *irho = dd->inv_rho_fluid + off;
      int fld = 0;
      if (type == AXG_DUMP_DISPL_VELO) {
        put_el(dd, fout, nef, e, fld++, chi + off);
        put_el(dd, fout, nef, e, fld++, dchi + off);
        continue;
      }
      if (type == AXG_DUMP_STRAIN_ONLY || type == AXG_DUMP_FULLFIELDS) {
        mat5 us, uz;
        grad_el(&s, axf[e], &w, chi + off, c1, c2);            /* usz = grad(chi) / rho */
        for (int k = 0; k < 25; ++k) {
          us[k] = c1[k] * (REAL)irho[k];
          uz[k] = c2[k] * (REAL)irho[k];
        }
        strain_el(&s, axf[e], &w, pole, 1, us, zero, uz, o);
        for (int q = 0; q < (nonmono ? 6 : 4); ++q) put_el(dd, fout, nef, e, fld++, o[q]);
      }
      if (type == AXG_DUMP_DISPL_ONLY || type == AXG_DUMP_FULLFIELDS) {
        grad_el(&s, axf[e], &w, type == AXG_DUMP_DISPL_ONLY ? chi + off : dchi + off, c1, c2);
        for (int k = 0; k < 25; ++k) {
          v3[0][k] = (REAL)irho[k] * c1[k];
          v3[2][k] = (REAL)irho[k] * c2[k];
        }
        put_el(dd, fout, nef, e, fld++, v3[0]);
        if (nonmono) put_el(dd, fout, nef, e, fld++, zero);
        put_el(dd, fout, nef, e, fld++, v3[2]);
      }
    }
    free(axf);
  }
  return ns + nf;
}
