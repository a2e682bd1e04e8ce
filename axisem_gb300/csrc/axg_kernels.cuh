// axg_kernels.cuh -- sm_103a kernels of the AxiSEM time loop.
//
// One CTA per patch of elements (axg_plan.h); one warp per element, one lane
// per GLL point (i, j) = (lane % 5, lane / 5), lanes 25..31 idle.  The 5x5
// tensor-product contractions of the reference (mxm_4 / vxm_4 of
// SOLVER/unrolled_loops.f90) are done with warp shuffles: lane (i, j) reads
// the five values of its column (k, j) or row (i, k) from the other lanes.
// Per-lane copies of the needed rows/columns of G1, G2 stay in registers.
//
// A patch kernel has three phases:
//   1. gather: the patch's global points are read once into shared memory
//      (time loop: the Newmark predictor is applied on the fly, so that the
//      arrays in HBM always hold the reference's state disp/velo/acc0);
//   2. elements, sub-round by sub-round: each warp computes its element's
//      stiffness and adds it into the shared point accumulators (elements
//      of one sub-round share no point, so there is no race);
//   3. write-back: the accumulators (which started from the partial sums of
//      earlier writers) are stored to the global force; the last writer of a
//      point applies the Newmark
//      corrector (SOLVER/time_evol_wave.F90:466-494) in registers and stores
//      disp/velo/acc0 -- the assembled force of that point never touches HBM.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "axg_plan.h"
#include "axg_tma.cuh"

namespace axg {

// Debug variant (-DAXG_DEVICE_CHECKS): every global and shared index is
// checked against its bound; the first violation is recorded in
// g_axg_check = {flag, kernel id, source line, 0, index lo, index hi, bound lo,
// bound hi} and the access is skipped.  Nothing traps.  Normal builds compile
// the checks away.
#ifdef AXG_DEVICE_CHECKS
__device__ int32_t g_axg_check[8];
__device__ __noinline__ bool axg_record(int kern, int line, long long idx, long long bound) {
  if (atomicCAS(&g_axg_check[0], 0, 1) == 0) {
    g_axg_check[1] = kern;
    g_axg_check[2] = line;
    g_axg_check[4] = (int32_t)(idx & 0xffffffff);
    g_axg_check[5] = (int32_t)(idx >> 32);
    g_axg_check[6] = (int32_t)(bound & 0xffffffff);
    g_axg_check[7] = (int32_t)(bound >> 32);
  }
  return false;
}
#define AXG_BOUND(idx, bound, kern)                                                          \
  ((((long long)(idx)) >= 0 && ((long long)(idx)) < ((long long)(bound)))                    \
       ? true                                                                               \
       : axg_record((kern), __LINE__, (long long)(idx), (long long)(bound)))
#else
#define AXG_BOUND(idx, bound, kern) true
#endif

constexpr int kWarps = 8;
constexpr int kThreads = 32 * kWarps;
constexpr unsigned kFull = 0xffffffffu;

enum { POLE_MONO = 0, POLE_DI = 1, POLE_QUAD = 2 };
// FORCE: stiffness + assembly; NEWMARK: a Newmark step
// (SOLVER/time_evol_wave.F90:264-502); SYMPLECTIC: one stage of a symplectic
// step (SOLVER/time_evol_wave.F90:516-742): drift u + c_d v on the gather,
// kick v + c_v a by the last writer
enum { MODE_FORCE = 0, MODE_NEWMARK = 1, MODE_SYMPLECTIC = 2 };

// slot of each metric array inside an element's block (same order as the
// host packing, SOLID_TERMS_USED of the Python mirror)
enum : int {
  S_M1 = 0, S_M2, S_M3, S_M4, S_MW1, S_M11S, S_M21S, S_M41S, S_M12S, S_M22S, S_M32S, S_M42S,
  S_M11Z, S_M21Z, S_M41Z,
  S_M5 = 15, S_M6, S_M7, S_M8, S_MW2, S_MW3,
  // dipole
  S_M13S = 21, S_M33S, S_M43S,
  // quadrupole
  S_MW4 = 21, S_MW5, S_M1PHI, S_M2PHI, S_M4PHI
};
__host__ __device__ constexpr int n_terms(int pole) { return pole == POLE_MONO ? 15 : (pole == POLE_DI ? 24 : 26); }
__host__ __device__ constexpr int n_axial(int pole) { return pole == POLE_MONO ? 3 : (pole == POLE_DI ? 9 : 6); }
__host__ __device__ constexpr int block_stride(int nt) { return ((nt * 25 + 3) / 4) * 4; }
// solid element block: nt*25 metric floats, then 25 uint16 patch-local point
// indices (50 bytes), 2 bytes pad, the int32 element info word; 16-byte multiple
__host__ __device__ constexpr int solid_idx_off(int nt) { return nt * 25; }      // in floats
__host__ __device__ constexpr int solid_info_off(int nt) { return nt * 25 + 13; }  // in floats
__host__ __device__ constexpr int solid_block_stride(int nt) { return ((nt * 25 + 14 + 3) / 4) * 4; }

struct SpecDev {
  float g1[25], g2[25], g0[5];
};

struct SrcTable {           // solid source points (<= 200)
  const int32_t *gidx;      // global point
  const float *val;         // (n, 3)
  const double *val_dp;     // (n, 3) in FP64, applied in FP64 by the compensated mode; or null
  int32_t n;
};

struct DomainArgs {
  const PatchMeta *meta;
  const uint32_t *pts;
  const int32_t *elinfo;    // bits 0..23: axial slot + 1; bits 24..27: source slot + 1
  const float *metric;      // per element block_stride(nt) floats (launch order)
  const float *m0;          // per axial slot n_axial*5 floats
  const float *fsmask;      // fluid free-surface mask per element (launch order) or null
  const float *srcfl;       // fluid element source terms (8, 25) or null
  const float *fx;          // solid, attenuation at every GLL point: per element (launch order) 3 x 25
                            // floats the Newmark step adds to the stiffness, or null
  int32_t patch_begin;
  int64_t n_patches, n_pts, n_elem, n_m0;   // buffer extents (checked builds)
};

struct StateArgs {
  float *u[3];              // disp (solid, gvec layout) / chi (fluid: u[0]); plain Newmark: the
                            // buffer the step stores the next step's prediction into
  float *v[3];              // velo / dchi
  float *a[3];              // acc0 / ddchi0
  float *f[3];              // force partial sums
  float *cu[3], *cv[3];     // compensated mode: running compensation of disp / velo (chi / dchi), else null
  float *up[3];             // plain Newmark: the step's predicted displacement (chi), which becomes its
                            // new displacement (the two buffers trade roles every step); else null
  const float *inv_mass;    // per global point
  const double *inv_mass_dp;  // per global point in FP64 (compensated mode) or null
  const float *gamma;       // absorbing gamma per global point or null
  const float *stf;         // (niter)
  const int32_t *iter;      // device iteration counter (1-based iter of this step)
  int32_t *blowup;          // first iteration that blew up (0 = none)
  int32_t *err;             // device error word (AXG_ERR_TIMEOUT when a bounded wait gave up)
  float thresh;             // 10 |magnitude|
  // Newmark: deltat, deltat/2, deltat^2/2; symplectic stage: dt = coefd(i) deltat,
  // kick = coefv(i) deltat; each an FP32 pair (value + _lo = the FP64 value)
  float dt, hdt, hdt2, dt_lo, hdt_lo, hdt2_lo;
  float kick, kick_lo;
  int32_t stage;            // 1 in a symplectic stage (the gathers drift), 0 in a Newmark step
  SrcTable src;
  int64_t nglob;            // extent of the state arrays (checked builds)
  int32_t niter;            // extent of stf
};

// ------------------------------------------------------------ work descriptors

// A launch's per-solve arguments, passed in its parameter space
// (__grid_constant__).  One<W>: one solve owns all of the launch's work items
// (a colour's patches, the boundary points, ...).  Many<W>: up to kMaxBatch
// solves advanced together by one launch; solve s owns the items
// [start[s], start[s + 1]), and a CTA or thread finds its solve from them.
constexpr int kMaxBatch = 32;

template <class W>
struct One {
  static constexpr bool kMany = false;
  W w;
  int32_t n_items;
  __device__ __forceinline__ int32_t items() const { return n_items; }
  __device__ __forceinline__ int locate(int32_t) const { return 0; }
  __device__ __forceinline__ int32_t first(int) const { return 0; }
  __device__ __forceinline__ const W &at(int) const { return w; }
};

template <class W>
struct Many {
  static constexpr bool kMany = true;
  int32_t n;                       // solves, 1..kMaxBatch
  int32_t start[kMaxBatch + 1];    // item prefix over the solves
  W w[kMaxBatch];
  __device__ __forceinline__ int32_t items() const { return start[n]; }
  __device__ __forceinline__ int locate(int32_t it) const {
    int s = 0;
    while (s + 1 < n && start[s + 1] <= it) ++s;
    return s;
  }
  __device__ __forceinline__ int32_t first(int s) const { return start[s]; }
  __device__ __forceinline__ const W &at(int s) const { return w[s]; }
};

// Attenuation data (cg4).
//
// Coarse-grained SLS attenuation: memory variables live at the four GLL
// points (1,1), (1,3), (3,1), (3,3) of every solid element, the lanes 6, 16,
// 8, 18 of the element's warp ("cg lanes", cg index k = 0..3 in that order,
// the order of the reference's (1:4) arrays).
//
// Per element (launch order) the host packs two arrays:
//   constants, kAnelConst floats: [field][k] for the fields below, then the
//     two Q-table rows (int32 bits) of Q_mu and Q_kappa;
//   state, anel_state_stride(n_sls) floats: memory_var_cg4(1:4,6,n_sls) in
//     the reference's order, src_tr_tm1(1:4), src_dev_tm1(1:4,6).
// Both travel with the element's metric block into the warp's ring; the
// updated state is written back from shared memory.
constexpr int kMaxSls = 8;
enum : int {
  A_DMU = 0, A_DKA = 4, A_Y = 8, A_VSE = 12, A_VSX = 16, A_VZE = 20, A_VZX = 24,
  A_DSDETA = 28, A_DZDETA = 32, A_DSDXI = 36, A_DZDXI = 40, A_INVS = 44, A_QMU = 48, A_QKA = 49
};
constexpr int kAnelConst = 52;  // floats, a 16-byte multiple
__host__ __device__ constexpr int anel_state_stride(int nsls) { return ((24 * nsls + 28 + 3) / 4) * 4; }
constexpr int kAnelSlot = kAnelConst + anel_state_stride(kMaxSls);  // floats per ring slot

struct AnelArgs {
  const float *consts;      // per element kAnelConst floats (launch order)
  float *state;             // per element state_stride floats (launch order)
  const float *qtab;        // per distinct Q: ts_fac_t(j) a_j(Q) at [0, kMaxSls), ts_fac_tm1(j) a_j(Q) after
  float ex[kMaxSls];        // exp_w_j_deltat
  int32_t nsls, state_stride, n_q;
};

// patch kernels: the domain (patch_begin = the colour's first patch) and state
struct PatchWork {
  DomainArgs d;
  StateArgs st;
};
// the attenuation data of the solves of an attenuated batch launch (the
// launch's Many<PatchWork> order)
struct AnelBatch {
  AnelArgs a[kMaxBatch];
};

// How a patch kernel's body sees its work items.  OneSolve refers to the
// kernel's own by-value parameters, so that the body reads them exactly as a
// kernel written for one solve does (as constant-bank operands); ManySolves
// indexes the batch's descriptors at run time.
struct OneSolve {
  static constexpr bool kMany = false;
  const DomainArgs &d;
  const StateArgs &st;
  int32_t n;
  const AnelArgs &an;
  __device__ __forceinline__ int32_t items() const { return n; }
  __device__ __forceinline__ int locate(int32_t) const { return 0; }
  __device__ __forceinline__ int32_t first(int) const { return 0; }
  __device__ __forceinline__ const DomainArgs &dom(int) const { return d; }
  __device__ __forceinline__ const StateArgs &state(int) const { return st; }
  __device__ __forceinline__ const AnelArgs *anel(int) const { return &an; }
};
struct ManySolves {
  static constexpr bool kMany = true;
  const Many<PatchWork> &m;
  const AnelArgs *an;  // per solve of the launch (attenuated batches), else null
  __device__ __forceinline__ int32_t items() const { return m.items(); }
  __device__ __forceinline__ int locate(int32_t it) const { return m.locate(it); }
  __device__ __forceinline__ int32_t first(int s) const { return m.first(s); }
  __device__ __forceinline__ const DomainArgs &dom(int s) const { return m.w[s].d; }
  __device__ __forceinline__ const StateArgs &state(int s) const { return m.w[s].st; }
  __device__ __forceinline__ const AnelArgs *anel(int s) const { return an + s; }
};

// ------------------------------------------------------------ small helpers

// Time-step coefficients as FP32 pairs.  The reference multiplies its FP32
// fields by FP64 coefficients (deltat, half_dt, half_dt_sq, coefd(i) and
// coefv(i) times deltat) and rounds each update once.  A coefficient rounded
// to FP32 is off by up to 3e-8 relative, the same in every step: over 1e5
// steps a steady drift of the solution's time scale, which the compensated
// summation cannot remove.  With the low part the increments carry only the
// FP32 rounding of the product.
// c x for the coefficient c + c_lo
__device__ __forceinline__ float mul2(float c, float c_lo, float x) { return fmaf(c, x, c_lo * x); }
// the predictor's increment deltat*velo + half_dt_sq*acc0
__device__ __forceinline__ float pred_inc(float v, float a, const StateArgs &st) {
  return fmaf(st.hdt2, a, fmaf(st.dt, v, fmaf(st.hdt2_lo, a, st.dt_lo * v)));
}
// disp + deltat*velo + half_dt_sq*acc0 (SOLVER/time_evol_wave.F90:357-364);
// a symplectic stage's drift disp + coefd(i) velo (hdt2 = 0)
__device__ __forceinline__ float predict(float d, float v, float a, const StateArgs &st) {
  return d + pred_inc(v, a, st);
}

// Compensated mode (no counterpart in the reference): x + inc by Kahan's
// compensated summation.  c carries the low-order part the previous additions
// lost; it is taken off the increment before the addition and replaced by
// what this addition loses, so that rounding does not accumulate over many
// steps.  (No fast-math: the compiler keeps (t - x) - y as written.)
__device__ __forceinline__ float kahan_add(float x, float inc, float &c) {
  const float y = inc - c;
  const float t = x + y;
  c = (t - x) - y;
  return t;
}
// components apply_axis_mask_{onecomp,twocomp,threecomp} zero on the axis
// (SOLVER/apply_masks.f90): s (monopole), phi and z (dipole), all (quadrupole)
template <int POLE>
__device__ __forceinline__ bool axis_masked(int comp) {
  return POLE == POLE_QUAD || (POLE == POLE_MONO ? comp == 0 : comp != 0);
}

// The predictor of the compensated mode: the increment's FP32 part, added by
// compensated summation.  Its low-coefficient part was taken off the stored
// compensation by the previous step's last writer (comp_after_step), so
// that the gathers, which hold many points' values at once, need no more
// registers than the increment takes.
__device__ __forceinline__ float predict_comp(float d, float v, float a, const StateArgs &st, float &c) {
  return kahan_add(d, fmaf(st.hdt2, a, st.dt * v), c);
}
// the compensation a last writer stores with the new state: c less the low
// part of the next predictor's increment deltat*velo + half_dt_sq*acc0
__device__ __forceinline__ float comp_after_step(float c, float v, float a, const StateArgs &st) {
  return c - fmaf(st.hdt2_lo, a, st.dt_lo * v);
}
// a symplectic stage's compensated drift disp + coefd(i) velo
__device__ __forceinline__ float drift_comp(float d, float v, const StateArgs &st, float &c) {
  return kahan_add(d, mul2(st.dt, st.dt_lo, v), c);
}

// X(i,j) = sum_k c[k] * v(k,j)   (v(k,j) held by lane k + 5 j)
__device__ __forceinline__ float dxi(float v, const float (&c)[5], int j5) {
  float s = c[0] * __shfl_sync(kFull, v, j5);
  s = fmaf(c[1], __shfl_sync(kFull, v, j5 + 1), s);
  s = fmaf(c[2], __shfl_sync(kFull, v, j5 + 2), s);
  s = fmaf(c[3], __shfl_sync(kFull, v, j5 + 3), s);
  s = fmaf(c[4], __shfl_sync(kFull, v, j5 + 4), s);
  return s;
}
// X(i,j) = sum_k v(i,k) * c[k]   (v(i,k) held by lane i + 5 k)
__device__ __forceinline__ float deta(float v, const float (&c)[5], int i) {
  float s = __shfl_sync(kFull, v, i) * c[0];
  s = fmaf(__shfl_sync(kFull, v, i + 5), c[1], s);
  s = fmaf(__shfl_sync(kFull, v, i + 10), c[2], s);
  s = fmaf(__shfl_sync(kFull, v, i + 15), c[3], s);
  s = fmaf(__shfl_sync(kFull, v, i + 20), c[4], s);
  return s;
}

// per-lane rows/columns of the derivative matrices (column-major G(a,b) = g[a+5b])
struct LaneCoef {
  float xi2[5], xi1[5];    // G2(k,i), G1(k,i): first stage d/dxi  (mxm_4(G2T,u))
  float eta[5];            // G2(k,j): first stage d/deta          (mxm_4(u,G2))
  float sxi2[5], sxi1[5];  // G2(i,k), G1(i,k): second stage       (mxm_4(G2,S))
  float seta[5];           // G2(j,k): second stage                (mxm_4(S,G2T))
  float g0i;               // G0(i)
  float g0[5];             // G0(k)
};

__device__ __forceinline__ void load_coef(const SpecDev &sp, int i, int j, LaneCoef &c) {
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    c.xi2[k] = sp.g2[k + 5 * i];
    c.xi1[k] = sp.g1[k + 5 * i];
    c.eta[k] = sp.g2[k + 5 * j];
    c.sxi2[k] = sp.g2[i + 5 * k];
    c.sxi1[k] = sp.g1[i + 5 * k];
    c.seta[k] = sp.g2[j + 5 * k];
    c.g0[k] = sp.g0[k];
  }
  c.g0i = sp.g0[i];
}

template <bool AX>
__device__ __forceinline__ const float (&cxi(const LaneCoef &c))[5] { return AX ? c.xi1 : c.xi2; }
template <bool AX>
__device__ __forceinline__ const float (&csxi(const LaneCoef &c))[5] { return AX ? c.sxi1 : c.sxi2; }

// element-local value of metric array `slot` at point `lane` (< 25); `blk` is
// the element's block staged in shared memory
__device__ __forceinline__ float ldm(const float *blk, int slot, int lane) { return blk[slot * 25 + lane]; }

// ------------------------------------------------------------ element stiffness

// glob_stiffness_mono_4 (SOLVER/stiffness_mono.f90:60-157) for lane (i, j)
// gx[c], ge[c] receive the first-stage derivatives d/dxi (mxm_4(G2T or G1T, u))
// and d/deta (mxm_4(u, G2)) of component c at the lane's point, the inputs of
// the cg4 strain (SOLVER/pointwise_derivatives.f90:216-250)
template <bool AX>
__device__ __forceinline__ void stiff_mono(const LaneCoef &c, const float *blk, const float *m0, int lane,
                                           int i, int j, float us, float uz, float &fs, float &fz,
                                           float (&gx)[3], float (&ge)[3]) {
  const int j5 = 5 * j;
  float X1 = dxi(us, cxi<AX>(c), j5);
  float X2 = dxi(uz, cxi<AX>(c), j5);
  float X3 = deta(us, c.eta, i);
  float X4 = deta(uz, c.eta, i);
  gx[0] = X1; gx[1] = 0.f; gx[2] = X2;
  ge[0] = X3; ge[1] = 0.f; ge[2] = X4;
  const float m1 = ldm(blk, S_M1, lane), m2 = ldm(blk, S_M2, lane), m3 = ldm(blk, S_M3, lane),
              m4 = ldm(blk, S_M4, lane), mw1 = ldm(blk, S_MW1, lane);
  const float m11s = ldm(blk, S_M11S, lane), m21s = ldm(blk, S_M21S, lane), m41s = ldm(blk, S_M41S, lane),
              m12s = ldm(blk, S_M12S, lane), m22s = ldm(blk, S_M22S, lane), m32s = ldm(blk, S_M32S, lane),
              m42s = ldm(blk, S_M42S, lane), m11z = ldm(blk, S_M11Z, lane), m21z = ldm(blk, S_M21Z, lane),
              m41z = ldm(blk, S_M41Z, lane);
  float ls = m4 * X4 + m2 * X3 + m1 * X1 + m3 * X2 + us * mw1;
  const float S1s = m11s * X3 + m21s * X1 + m12s * X4 + m22s * X2 + m1 * us;
  const float S2s = m11s * X1 + m41s * X3 + m32s * X2 + m42s * X4 + m2 * us;
  const float S1z = m11z * X4 + m21z * X2 + m32s * X3 + m22s * X1 + m3 * us;
  const float S2z = m11z * X2 + m41z * X4 + m12s * X1 + m42s * X3 + m4 * us;
  X2 = deta(S2s, c.seta, i);
  X4 = deta(S2z, c.seta, i);
  X1 = dxi(S1s, csxi<AX>(c), j5);
  X3 = dxi(S1z, csxi<AX>(c), j5);
  ls = ls + X1 + X2;
  float lz = X3 + X4;
  if (AX) {
    const float w1 = m0[0 * 5 + j], w2 = m0[1 * 5 + j], w3 = m0[2 * 5 + j];
    float V1 = dxi(us, c.g0, j5);   // vxm_4(G0, us)
    float V2 = deta(uz, c.eta, 0);  // vxm_4(uz(0,:), G2)
    float V4 = w1 * V1 + w3 * V2;
    const float V3 = dxi(uz, c.g0, j5);
    V4 = V4 + w2 * V3;
    float Xa = c.g0i * (w2 * V1);
    const float V2b = w3 * V1;
    const float V1b = deta(V2b, c.seta, 0);  // vxm_4(V2, G2T)
    if (i == 0) Xa = Xa + V1b;
    ls = ls + c.g0i * V4;
    lz = Xa + lz;
  }
  fs = ls;
  fz = lz;
}

// glob_stiffness_di_4 (SOLVER/stiffness_di.f90:60-256)
template <bool AX>
__device__ __forceinline__ void stiff_di(const LaneCoef &c, const float *blk, const float *m0, int lane, int i,
                                         int j, float u1, float u2, float u3, float &f1, float &f2, float &f3,
                                         float (&gx)[3], float (&ge)[3]) {
  const int j5 = 5 * j;
  float X4 = deta(u1, c.eta, i), X5 = deta(u2, c.eta, i), X6 = deta(u3, c.eta, i);
  float X1 = dxi(u1, cxi<AX>(c), j5), X2 = dxi(u2, cxi<AX>(c), j5), X3 = dxi(u3, cxi<AX>(c), j5);
  gx[0] = X1; gx[1] = X2; gx[2] = X3;
  ge[0] = X4; ge[1] = X5; ge[2] = X6;
  const float X7 = X1 + X2, X8 = X4 + X5;
  const float m1 = ldm(blk, S_M1, lane), m2 = ldm(blk, S_M2, lane), m3 = ldm(blk, S_M3, lane),
              m4 = ldm(blk, S_M4, lane), m5 = ldm(blk, S_M5, lane), m6 = ldm(blk, S_M6, lane),
              m7 = ldm(blk, S_M7, lane), m8 = ldm(blk, S_M8, lane);
  const float mw1 = ldm(blk, S_MW1, lane), mw2 = ldm(blk, S_MW2, lane), mw3 = ldm(blk, S_MW3, lane);
  const float m11s = ldm(blk, S_M11S, lane), m21s = ldm(blk, S_M21S, lane), m41s = ldm(blk, S_M41S, lane),
              m12s = ldm(blk, S_M12S, lane), m22s = ldm(blk, S_M22S, lane), m42s = ldm(blk, S_M42S, lane),
              m13s = ldm(blk, S_M13S, lane), m23s = ldm(blk, S_M32S, lane), m33s = ldm(blk, S_M33S, lane),
              m43s = ldm(blk, S_M43S, lane), m11z = ldm(blk, S_M11Z, lane), m21z = ldm(blk, S_M21Z, lane),
              m41z = ldm(blk, S_M41Z, lane);
  const float ls2 = m8 * X6 + m7 * X3 + m1 * X1 + m5 * X2 + m2 * X4 + m6 * X5 + mw1 * u2 + mw2 * u3;
  const float ls3 = m4 * X4 - m4 * X5 + m3 * X1 - m3 * X2 + mw2 * u2 + mw3 * u3;
  float c1 = m13s * X6, c2 = m23s * X3, c3 = m3 * u3;
  float s1p = c1 + c2 + c3 + m11s * X4 + m21s * X1 + m12s * X5 + m22s * X2 + m1 * u2;
  float s1m = c1 + c2 - c3 + m11s * X5 + m21s * X2 + m12s * X4 + m22s * X1 + m5 * u2;
  c1 = m33s * X3;
  c2 = m43s * X6;
  c3 = m4 * u3;
  const float s2p = c1 + c2 + c3 + m11s * X1 + m41s * X4 + m12s * X2 + m42s * X5 + m2 * u2;
  const float s2m = c1 + c2 - c3 + m11s * X2 + m41s * X5 + m12s * X1 + m42s * X4 + m6 * u2;
  float S1z = m33s * X8 + m23s * X7 + m11z * X6 + m21z * X3 + m7 * u2;
  const float S2z = m13s * X7 + m43s * X8 + m11z * X3 + m41z * X6 + m8 * u2;
  X1 = dxi(s1p, csxi<AX>(c), j5);
  X3 = dxi(s1m, csxi<AX>(c), j5);
  X5 = dxi(S1z, csxi<AX>(c), j5);
  X2 = deta(s2p, c.seta, i);
  X4 = deta(s2m, c.seta, i);
  X6 = deta(S2z, c.seta, i);
  float l1 = X1 + X2;
  float l2 = X3 + X4 + ls2;
  float l3 = X5 + X6 + ls3;
  if (AX) {
    // M0_w slots: 0:w1 1:w2 2:w3 3:w4 4:w6 5:w7 6:w8 7:w9 8:w10
    const float w1 = m0[0 * 5 + j], w2 = m0[1 * 5 + j], w3 = m0[2 * 5 + j], w4 = m0[3 * 5 + j],
                w6 = m0[4 * 5 + j], w7 = m0[5 * 5 + j], w8 = m0[6 * 5 + j], w9 = m0[7 * 5 + j],
                w10 = m0[8 * 5 + j];
    const float V1 = dxi(u1, c.g0, j5), V2 = dxi(u2, c.g0, j5), V3 = dxi(u3, c.g0, j5);
    const float V4 = deta(u1, c.eta, 0), V5 = deta(u2, c.eta, 0);
    (void)V5;
    const float a_p = w1 * V2 + w3 * V3;
    const float a_m = w1 * V1 + (w2 + w6) * V4 + w9 * V2 + w10 * V3;
    const float a_z = w3 * V1 + (w4 + w8) * V4 + w7 * V3 + w10 * V2;
    float S1p = c.g0i * a_p;
    const float S1m = c.g0i * a_m;
    S1z = c.g0i * a_z;
    const float V4b = (w2 + w6) * V2 + (w4 + w8) * V3;
    const float V1b = deta(V4b, c.seta, 0);
    if (i == 0) S1p = S1p + V1b;
    l1 = l1 + S1p;
    l2 = l2 + S1m;
    l3 = l3 + S1z;
  }
  f1 = l1;
  f2 = l2;
  f3 = l3;
}

// glob_stiffness_quad_4 (SOLVER/stiffness_quad.f90:238-414)
template <bool AX>
__device__ __forceinline__ void stiff_quad(const LaneCoef &c, const float *blk, const float *m0, int lane,
                                           int i, int j, float us, float up, float uz, float &f1, float &f2,
                                           float &f3, float (&gx)[3], float (&ge)[3]) {
  const int j5 = 5 * j;
  float X1 = dxi(us, cxi<AX>(c), j5), X2 = dxi(up, cxi<AX>(c), j5), X3 = dxi(uz, cxi<AX>(c), j5);
  float X4 = deta(us, c.eta, i), X5 = deta(up, c.eta, i), X6 = deta(uz, c.eta, i);
  gx[0] = X1; gx[1] = X2; gx[2] = X3;
  ge[0] = X4; ge[1] = X5; ge[2] = X6;
  const float m1 = ldm(blk, S_M1, lane), m2 = ldm(blk, S_M2, lane), m3 = ldm(blk, S_M3, lane),
              m4 = ldm(blk, S_M4, lane), m5 = ldm(blk, S_M5, lane), m6 = ldm(blk, S_M6, lane),
              m7 = ldm(blk, S_M7, lane), m8 = ldm(blk, S_M8, lane);
  const float mw1 = ldm(blk, S_MW1, lane), mw2 = ldm(blk, S_MW2, lane), mw3 = ldm(blk, S_MW3, lane),
              mw4 = ldm(blk, S_MW4, lane), mw5 = ldm(blk, S_MW5, lane);
  const float m11s = ldm(blk, S_M11S, lane), m21s = ldm(blk, S_M21S, lane), m41s = ldm(blk, S_M41S, lane),
              m12s = ldm(blk, S_M12S, lane), m22s = ldm(blk, S_M22S, lane), m32s = ldm(blk, S_M32S, lane),
              m42s = ldm(blk, S_M42S, lane), m11z = ldm(blk, S_M11Z, lane), m21z = ldm(blk, S_M21Z, lane),
              m41z = ldm(blk, S_M41Z, lane), m1p = ldm(blk, S_M1PHI, lane), m2p = ldm(blk, S_M2PHI, lane),
              m4p = ldm(blk, S_M4PHI, lane);
  const float c1 = m2 * X4, c2 = m1 * X1, c3 = m6 * X5, c4 = m5 * X2, c5 = m4 * X6, c6 = m3 * X3;
  float ls = c1 + c2 + 2.f * (c3 + c4) + c5 + c6 + mw1 * us + mw2 * up + 2.f * mw3 * uz;
  float lp = -2.f * (c1 + c2 + c5 + c6) - (c3 + c4) + mw2 * us + mw4 * up - mw3 * uz;
  float lz = 2.f * (m8 * X5 + m7 * X2) + mw3 * (2.f * us - up) + mw5 * uz;
  const float usm = us - 2.f * up, ups = 2.f * us - up;
  const float S1s = m11s * X4 + m21s * X1 + m12s * X6 + m22s * X3 + m1 * usm;
  const float S2s = m11s * X1 + m41s * X4 + m32s * X3 + m42s * X6 + m2 * usm;
  const float S1z = m11z * X6 + m21z * X3 + m32s * X4 + m22s * X1 + m3 * usm;
  const float S2z = m11z * X3 + m41z * X6 + m12s * X1 + m42s * X4 + m4 * usm;
  const float S1p = m1p * X5 + m2p * X2 + m5 * ups + 2.f * m7 * uz;
  const float S2p = m1p * X2 + m4p * X5 + m6 * ups + 2.f * m8 * uz;
  X2 = deta(S2s, c.seta, i);
  X4 = deta(S2p, c.seta, i);
  X6 = deta(S2z, c.seta, i);
  X1 = dxi(S1s, csxi<AX>(c), j5);
  X3 = dxi(S1p, csxi<AX>(c), j5);
  X5 = dxi(S1z, csxi<AX>(c), j5);
  ls = ls + X1 + X2;
  lp = lp + X3 + X4;
  lz = lz + X5 + X6;
  if (AX) {
    const float w1 = m0[0 * 5 + j], w2 = m0[1 * 5 + j], w3 = m0[2 * 5 + j], w4 = m0[3 * 5 + j],
                w5 = m0[4 * 5 + j], w6 = m0[5 * 5 + j];
    const float V1 = dxi(us, c.g0, j5), V2 = dxi(up, c.g0, j5), V3 = dxi(uz, c.g0, j5);
    ls = ls + c.g0i * (w1 * V1 + w2 * V2 + w3 * V3);
    lp = lp + c.g0i * (w2 * V1 + w4 * V2 + w5 * V3);
    lz = lz + c.g0i * (w3 * V1 + w5 * V2 + w6 * V3);
  }
  f1 = ls;
  f2 = lp;
  f3 = lz;
}

// ------------------------------------------------------------ attenuation (cg4)

// Lanes 0..23: memory-variable entry (component lane / 4, cg point lane % 4)
// of the state R summed over the n_sls solids (the sum the anelastic
// stiffness takes); other lanes 0.
__device__ __forceinline__ float memvar_sum(const float *R, int nsls, int lane) {
  float rs = 0.f;
  if (lane < 24)
    for (int q = 0; q < nsls; ++q) rs = rs + R[q * 24 + lane];
  return rs;
}

// Anelastic stiffness (glob_anel_stiffness_{mono,di,quad}_cg4,
// SOLVER/stiffness_mono.f90:511, SOLVER/stiffness_di.f90:727,
// SOLVER/stiffness_quad.f90:672) for lane (i, j): subtracts the divergence of
// the summed memory-variable stress from f.  The sparse products
// mxm_cg4_sparse_b(G, S1) and mxm_cg4_sparse_a(S2, G2T) of
// SOLVER/unrolled_loops.f90 become two shuffles each: X1(i,j) for j in {1,3}
// takes S1 at (1,j), (3,j); X2(i,j) for i in {1,3} takes S2 at (i,1), (i,3).
template <int POLE, bool AX>
__device__ __forceinline__ void anel_stiffness(const LaneCoef &c, const float *cs, float rs, bool cg, int k, int i,
                                               int j, bool active, int lane, float &f0, float &f1, float &f2) {
  float S1a = 0.f, S2a = 0.f, S1b = 0.f, S2b = 0.f, S1z = 0.f, S2z = 0.f;
  float ya = 0.f, yb = 0.f, yz = 0.f;
  // rs: lanes 0..23 hold entry (component lane / 4, cg point lane % 4)
  // summed over the SLS (memvar_sum); cg lane k collects its six components
  float r[6];
#pragma unroll
  for (int v = 0; v < 6; ++v) r[v] = __shfl_sync(kFull, rs, (v * 4 + k) & 31);
  if (cg) {
    const float vse = cs[A_VSE + k], vsx = cs[A_VSX + k], vze = cs[A_VZE + k], vzx = cs[A_VZX + k];
    const float yl = cs[A_Y + k];
    if (POLE == POLE_DI) {
      S1a = vze * (r[0] - r[5]) + vse * (r[4] - r[3]);
      S2a = vzx * (r[0] - r[5]) + vsx * (r[4] - r[3]);
      S1b = vze * (r[0] + r[5]) + vse * (r[4] + r[3]);
      S2b = vzx * (r[0] + r[5]) + vsx * (r[4] + r[3]);
    } else {
      S1a = vze * r[0] + vse * r[4];
      S2a = vzx * r[0] + vsx * r[4];
      if (POLE == POLE_QUAD) {
        S1b = vze * r[5] + vse * r[3];
        S2b = vzx * r[5] + vsx * r[3];
      }
    }
    S1z = vze * r[4] + vse * r[2];
    S2z = vzx * r[4] + vsx * r[2];
    if (POLE == POLE_MONO) {
      ya = yl * r[1];
    } else if (POLE == POLE_DI) {
      yb = 2.f * yl * (r[1] - r[5]);
      yz = -(yl * r[3]);
    } else {
      ya = yl * (r[1] - 2.f * r[5]);
      yb = yl * (r[5] - 2.f * r[1]);
      yz = -(2.f * yl * r[3]);
    }
  }
  const bool jc = active && (j == 1 || j == 3), ic = active && (i == 1 || i == 3);
  const int sj1 = 1 + 5 * j, sj3 = 3 + 5 * j, si1 = i + 5, si3 = i + 15;
  const float gi1 = csxi<AX>(c)[1], gi3 = csxi<AX>(c)[3];  // G(i,1), G(i,3); G = G1 on axial elements
  const float g1j = c.seta[1], g3j = c.seta[3];            // G2T(1,j), G2T(3,j)
  auto x1 = [&](float S) {
    const float p = __shfl_sync(kFull, S, sj1), q = __shfl_sync(kFull, S, sj3);
    return jc ? gi1 * p + gi3 * q : 0.f;
  };
  auto x2 = [&](float S) {
    const float p = __shfl_sync(kFull, S, si1), q = __shfl_sync(kFull, S, si3);
    return ic ? p * g1j + q * g3j : 0.f;
  };
  const float la = x1(S1a) + x2(S2a) + ya;
  const float lz = x1(S1z) + x2(S2z) + yz;
  f0 = f0 - la;
  f2 = f2 - lz;
  if (POLE == POLE_DI) {
    const float lb = x1(S1b) + x2(S2b) + yb;
    f1 = f1 - lb;
  } else if (POLE == POLE_QUAD) {
    const float lb = (-x1(S1b) - x2(S2b)) + yb;
    f1 = f1 - lb;
  }
}

// Memory-variable time step of an element (time_step_memvars_cg4,
// SOLVER/attenuation.f90:81-202) with the strain of
// compute_strain_att_el_cg4 (:471-535).  The four cg lanes form the strain
// at their point: gx, ge are the lane's first-stage derivatives d/dxi,
// d/deta of the three displacement components, u its (predicted,
// axis-masked) displacement; the gradient at a cg point is
// axisym_gradient_solid_el_cg4 (SOLVER/pointwise_derivatives.f90:216-250),
// f/s is f_over_s_solid_el_cg4 (:55-75) with the stored 1/s.  They leave the
// step's sources in `scr` (src_dev(v,k) at 4v+k, src_tr(k) at 24+k); then
// every lane of the warp updates memory variables R(k,v,j) (entry
// 24j + 4v + k) in place, and the sources become the previous step's.
template <int POLE>
__device__ __forceinline__ float anel_memvar_step(const float *cs, float *R, float *scr, const AnelArgs &an, bool cg,
                                                  int k, int lane, const float (&u)[3], const float (&gx)[3],
                                                  const float (&ge)[3]) {
  const int nsls = an.nsls;
  float *trm1 = R + 24 * nsls, *dm1 = trm1 + 4;
  if (cg) {
    const float dsdeta = cs[A_DSDETA + k], dzdeta = cs[A_DZDETA + k];
    const float dsdxi = cs[A_DSDXI + k], dzdxi = cs[A_DZDXI + k], invs = cs[A_INVS + k];
    auto grad_s = [&](float m1, float m2) { return dzdeta * m1 + dzdxi * m2; };
    auto grad_z = [&](float m1, float m2) { return dsdeta * m1 + dsdxi * m2; };
    float g[6];
    float b1x = gx[0], b1e = ge[0];
    if (POLE == POLE_DI) {
      b1x = gx[0] + gx[1];
      b1e = ge[0] + ge[1];
    }
    const float b1s = grad_s(b1x, b1e), b1z = grad_z(b1x, b1e);
    const float b2s = grad_s(gx[2], ge[2]), b2z = grad_z(gx[2], ge[2]);
    g[0] = b1s;
    g[2] = b2z;
    g[4] = b1z + b2s;
    if (POLE == POLE_MONO) {
      g[1] = invs * u[0];
      g[3] = 0.f;
      g[5] = 0.f;
    } else if (POLE == POLE_DI) {
      g[1] = 2.f * (invs * u[1]);
      const float cx = gx[0] - gx[1], ce = ge[0] - ge[1];
      g[3] = -(invs * u[2]) - grad_z(cx, ce);
      g[5] = -g[1] - grad_s(cx, ce);
    } else {
      g[1] = invs * (u[0] - 2.f * u[1]);
      g[3] = -2.f * (invs * u[2]) - grad_z(gx[1], ge[1]);
      g[5] = invs * (u[1] - 2.f * u[0]) - grad_s(gx[1], ge[1]);
    }
    const float tr = g[0] + g[1] + g[2];
    const float dm = cs[A_DMU + k];
#pragma unroll
    for (int v = 0; v < 3; ++v) scr[4 * v + k] = (dm * 2.f) * (g[v] - tr * (1.f / 3.f));
    scr[12 + k] = POLE == POLE_MONO ? 0.f : dm * g[3];
    scr[16 + k] = dm * g[4];
    scr[20 + k] = POLE == POLE_MONO ? 0.f : dm * g[5];
    scr[24 + k] = cs[A_DKA + k] * tr;
  }
  __syncwarp();
  int qmu = __float_as_int(cs[A_QMU]), qka = __float_as_int(cs[A_QKA]);
  if (!AXG_BOUND(qmu, an.n_q, 4)) qmu = 0;
  if (!AXG_BOUND(qka, an.n_q, 4)) qka = 0;
  const float *tmu = an.qtab + qmu * 2 * kMaxSls, *tka = an.qtab + qka * 2 * kMaxSls;
  // lane = entry (component v, cg point kk) of every solid q; the sum of
  // the entries before the update is returned for the anelastic stiffness
  float rs = 0.f;
  if (lane < 24) {
    const int vk = lane, v = vk >> 2, kk = vk & 3;
    const bool upd = !(POLE == POLE_MONO && (v == 3 || v == 5));  // never written for the monopole
    const float sv = scr[vk], dv = dm1[vk], sk = scr[24 + kk], tk = trm1[kk];
    for (int q = 0; q < nsls; ++q) {
      const int e = q * 24 + vk;
      const float old = R[e];
      rs = rs + old;
      if (upd) {
        const float db = __ldg(tmu + q) * sv + __ldg(tmu + kMaxSls + q) * dv;
        float nv = an.ex[q] * old + db;
        if (v < 3) nv = nv + (__ldg(tka + q) * sk + __ldg(tka + kMaxSls + q) * tk);
        R[e] = nv;
      }
    }
  }
  __syncwarp();
  if (lane < 4) trm1[lane] = scr[24 + lane];
  else if (lane < 28) dm1[lane - 4] = scr[lane - 4];
  return rs;
}

// ------------------------------------------------------------ solid patch kernel

constexpr int kStages = 2;  // element blocks in flight per warp (TMA ring depth)

// shared-memory layout of the solid kernel (bytes); NB buffers of the patch
// state (u, f, point words), STG ring stages per warp, AS floats of
// attenuation data per stage (0 without attenuation)
template <int NC, int BS, int STG, int AS, int NB, int ROW, bool KAHAN>
struct SolidSmem {
  static constexpr int u_bytes = NC * ROW * 4, w_bytes = kMaxPatchPoints * 4;
  static constexpr int u_off = 0;
  static constexpr int f_off = u_off + NB * u_bytes;
  static constexpr int c_off = f_off + NB * u_bytes;  // compensated mode: predictor compensation
  static constexpr int w_off = c_off + (KAHAN ? u_bytes : 0);
  static constexpr int ring_off = ((w_off + NB * w_bytes + 127) / 128) * 128;
  static constexpr int aring_off = ring_off + kWarps * STG * BS * 4;
  static constexpr int scr_off = aring_off + kWarps * STG * AS * 4;     // attenuation: 32 floats per warp
  static constexpr int bar_off = scr_off + (AS > 0 ? kWarps * 32 * 4 : 0);
  static constexpr int bytes = bar_off + kWarps * STG * 8;
};
// ring depth (the same with attenuation, whose blocks ride in a second ring)
__host__ __device__ constexpr int solid_stages(bool) { return kStages; }
// The gather is asynchronous (cp.async into shared memory, the next patch's
// during the current one's element rounds) where it only copies: the
// stiffness mode's u, and the plain elastic Newmark step's predicted
// displacement, which the previous step's last writers stored (up).  The
// others compute on the way in (the compensated predictor, a symplectic
// drift) or have no shared memory left for a second buffer (attenuation), and
// gather through registers.
__host__ __device__ constexpr bool solid_async(int mode, bool anel, bool kahan) {
  return mode == MODE_FORCE || (mode == MODE_NEWMARK && !anel && !kahan);
}
// patch-state buffers: two for the asynchronous gather
__host__ __device__ constexpr int solid_buffers(int mode, bool anel, bool kahan) {
  return solid_async(mode, anel, kahan) ? 2 : 1;
}
// resident CTAs per SM the kernel is compiled for: the plain elastic
// symplectic stage keeps three (its register-staged gather is latency-bound;
// 80 registers), the others two (no spills at 128 registers; two patch
// buffers fit)
__host__ __device__ constexpr int solid_min_ctas(int mode, bool anel, bool kahan = false) {
  return mode == MODE_SYMPLECTIC && !anel && !kahan ? 3 : 2;
}
// Bank swizzle of the shared point arrays: patch point t lives at
// t + pad * (t / 32).  An element's 25 points sit in five runs of five
// consecutive patch points, one run per element row; on structured blocks
// the runs lie a patch width (33 for 8 x 8 patches) apart, so unpadded they
// share only 9 of the 32 banks (5-way conflicts), padded by 4 words per 32
// they fall on 25 distinct banks.  The three-CTA elastic symplectic kernel
// can only afford 2 words per 32 (banks i + 3j: at most 2-way conflicts).
__host__ __device__ constexpr int solid_pad(int mode, bool anel, bool kahan = false) {
  return solid_min_ctas(mode, anel, kahan) == 2 ? 4 : 2;
}
__host__ __device__ constexpr int solid_row(int mode, bool anel, bool kahan = false) {
  return kMaxPatchPoints + solid_pad(mode, anel, kahan) * ((kMaxPatchPoints + 31) / 32);
}

// the sub-round ends of a patch held in registers (8 bits per round), so
// that no per-patch array is indexed at run time: a PatchMeta indexed that
// way lives in local memory, and each lookup is a local load
struct PatchRounds {
  uint64_t lo;  // round_end[0..7]
  uint32_t hi;  // round_end[8..11]
  int n;
  __device__ __forceinline__ explicit PatchRounds(const PatchMeta &m) : lo(0), hi(0), n(m.n_rounds) {
    static_assert(kMaxSubrounds <= 12, "PatchRounds holds 12 rounds");
#pragma unroll
    for (int r = 0; r < 8; ++r) lo |= (uint64_t)m.round_end[r] << (8 * r);
#pragma unroll
    for (int r = 0; r < 4; ++r) hi |= (uint32_t)m.round_end[8 + r] << (8 * r);
  }
  __device__ __forceinline__ int end(int r) const {
    return r < 8 ? (int)((lo >> (8 * r)) & 0xFFu) : (int)((hi >> (8 * (r - 8))) & 0xFFu);
  }
};

// the elements warp `w` processes in a patch, in order: sub-round by
// sub-round, elements w, w + kWarps, ... of each round
struct WarpIter {
  int r, s;
  __device__ __forceinline__ void norm(const PatchRounds &m, int w) {
    while (r < m.n && s >= m.end(r)) {
      ++r;
      s = m.end(r - 1) + w;
    }
  }
  __device__ __forceinline__ bool valid(const PatchRounds &m) const { return r < m.n; }
};

// ANEL (time loop only): attenuation of the solid, the anelastic stiffness
// before the axis mask of acc1 and the memory-variable step after it, as in
// SOLVER/time_evol_wave.F90 (anel_true, cg4).
// KAHAN (time loop only): compensated summation of the predictor and the
// velocity corrector (kahan_add); the predictor's new compensation travels
// from the gather to the last writer in shared memory.
template <int POLE, int MODE, bool ANEL, bool KAHAN, class P>
__device__ __forceinline__ void solid_patch_body(const P &p, const SpecDev &sp) {
  static_assert(!ANEL || MODE != MODE_FORCE, "attenuation runs in a time loop");
  static_assert(!P::kMany || MODE != MODE_FORCE, "batches run time-loop steps");
  static_assert(!KAHAN || MODE != MODE_FORCE, "the compensated mode is a time-loop mode");
  constexpr bool TL = MODE != MODE_FORCE;  // a time-loop mode
  constexpr int NC = POLE == POLE_MONO ? 2 : 3;           // stored components
  constexpr int NT = n_terms(POLE), NA = n_axial(POLE);
  constexpr int BS = solid_block_stride(NT);
  constexpr uint32_t BSB = BS * 4;
  constexpr int STG = solid_stages(ANEL);
  constexpr int AS = ANEL ? kAnelSlot : 0;
  constexpr int NB = solid_buffers(MODE, ANEL, KAHAN);
  constexpr bool ASYNC = solid_async(MODE, ANEL, KAHAN);
  // plain Newmark: the gather reads the predicted displacement (up), and the
  // last writers store the next step's
  constexpr bool LOOK = MODE == MODE_NEWMARK && !KAHAN;
  constexpr int ROW = solid_row(MODE, ANEL, KAHAN), PAD = solid_pad(MODE, ANEL, KAHAN);
  using L = SolidSmem<NC, BS, STG, AS, NB, ROW, KAHAN>;
  extern __shared__ __align__(128) unsigned char smem[];
  auto su_of = [&](int b) { return reinterpret_cast<float(*)[ROW]>(smem + L::u_off + b * L::u_bytes); };
  auto sf_of = [&](int b) { return reinterpret_cast<float(*)[ROW]>(smem + L::f_off + b * L::u_bytes); };
  float(*s_cu)[ROW] = reinterpret_cast<float(*)[ROW]>(smem + L::c_off);  // compensated mode only
  auto spos = [](int t) { return t + PAD * (t >> 5); };  // swizzled position of patch point t
  auto sw_of = [&](int b) { return reinterpret_cast<uint32_t *>(smem + L::w_off + b * L::w_bytes); };
  float *ring = reinterpret_cast<float *>(smem + L::ring_off);
  float *aring = reinterpret_cast<float *>(smem + L::aring_off);
  float *scr = reinterpret_cast<float *>(smem + L::scr_off);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L::bar_off);
  __shared__ int s_stop;
  __shared__ int s_timeout;  // a bounded wait of this CTA gave up
  // sub-round r of a patch is complete when all threads have arrived on
  // s_round[r] after their accumulations of round r
  __shared__ __align__(8) uint64_t s_round[kMaxSubrounds];
  __shared__ __align__(8) uint64_t s_wbar[2];  // a patch's point words have landed in buffer b
  // component c of the shared arrays -> global component (mono: s, z)
  auto gc = [](int c) { return (POLE == POLE_MONO && c == 1) ? 2 : c; };

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x < kWarps * STG) mbar_init(&bars[threadIdx.x], 1);
  if (threadIdx.x < kMaxSubrounds) mbar_init(&s_round[threadIdx.x], kThreads);
  if (threadIdx.x < 2) mbar_init(&s_wbar[threadIdx.x], 1);
  pdl_wait();  // the step's earlier kernels are complete
  // one solve: nothing to do after a blow-up (a batch checks per solve below)
  if (threadIdx.x == 0) s_stop = TL && !P::kMany ? *p.state(0).blowup : 0;
  if (threadIdx.x == 0) s_timeout = 0;
  fence_mbar_init();
  __syncthreads();
  if (s_stop) return;  // uniform across the CTA; no copy has been issued
  // the step's source time function value (a batch reads it per solve below)
  float stf_one = 0.f;
  if (TL && !P::kMany && AXG_BOUND(*p.state(0).iter - 1, p.state(0).niter, 3))
    stf_one = p.state(0).stf[*p.state(0).iter - 1];

  const bool active = lane < 25;
  const int i = lane % 5, j = active ? lane / 5 : 0;
  // idle lanes 25..31 take part in the shuffles; their reads of an element's
  // data go to point 24 so that no lane reads past the element's block
  const int ml = active ? lane : 24;
  LaneCoef coef;
  load_coef(sp, i, j, coef);
  const uint64_t pol = policy_evict_first();
  float *my_ring = ring + warp * STG * BS;
  float *my_aring = aring + warp * STG * AS;
  uint64_t *my_bars = bars + warp * STG;
  uint32_t kcount = 0;  // elements this warp has consumed (slot = kcount % STG)
  uint32_t round_par = 0;  // bit r: parity of the next completion of s_round[r]
  uint32_t pcount = 0;     // patches this CTA has started: buffer pcount % NB, s_wbar parity (pcount / NB) & 1
  // cg lane index k of the attenuation points (1,1), (1,3), (3,1), (3,3)
  const bool cg = active && (i == 1 || i == 3) && (j == 1 || j == 3);
  const int kcg = 2 * (i >> 1) + (j >> 1);
  // one thread: start the copies of element `el` of domain d (attenuation
  // data an) into ring slot `slot`
  auto issue = [&](const DomainArgs &d, const AnelArgs *an, uint32_t slot, int64_t el) {
    if (ANEL) {
      const uint32_t state_bytes = (uint32_t)an->state_stride * 4u;
      mbar_expect_tx(&my_bars[slot], BSB + kAnelConst * 4 + state_bytes);
      bulk_g2s_tx(my_ring + slot * BS, d.metric + el * BS, BSB, &my_bars[slot], pol);
      bulk_g2s_tx(my_aring + slot * AS, an->consts + el * kAnelConst, kAnelConst * 4, &my_bars[slot], pol);
      bulk_g2s_tx(my_aring + slot * AS + kAnelConst, an->state + el * an->state_stride, state_bytes, &my_bars[slot],
                  pol);
    } else {
      bulk_g2s(my_ring + slot * BS, d.metric + el * BS, BSB, &my_bars[slot], pol);
    }
  };
  // one thread: bulk copy of a patch's point words into buffer b (each
  // patch's words start 16-byte aligned, padded to a multiple of four)
  auto issue_words = [&](const DomainArgs &d, int b, int32_t pt_start, int n_pts) {
    const uint32_t nw = ((uint32_t)n_pts + 3u) & ~3u;
    if (nw > 0 && AXG_BOUND((int64_t)pt_start + nw - 1, d.n_pts, 1)) {
      fence_proxy_async();  // earlier generic reads of the buffer precede the async-proxy write
      bulk_g2s(sw_of(b), d.pts + pt_start, nw * 4u, &s_wbar[b], pol);
    } else {
      mbar_arrive(&s_wbar[b]);
    }
  };
  // every thread (asynchronous gather): 4-byte copies of its points' u (the
  // predicted displacement up in a Newmark step), and of the partial sums of
  // points an earlier writer (earlier colour, coupling pre-pass) holds,
  // straight into buffer b.  A point's accumulator starts from that partial
  // sum, so that the write-back is a plain store.
  auto issue_gather = [&](const StateArgs &st, int b, int n_pts) {
    float *const *src = MODE == MODE_NEWMARK ? st.up : st.u;
    float(*gu)[ROW] = su_of(b);
    float(*gf)[ROW] = sf_of(b);
    const uint32_t *gw = sw_of(b);
    for (int t = threadIdx.x; t < n_pts; t += kThreads) {
      const uint32_t w = gw[t];
      const uint32_t g = w & kPtIndexMask;
      const int pt = spos(t);
      if (!AXG_BOUND(g, st.nglob, 1)) {
#pragma unroll
        for (int c = 0; c < NC; ++c) gu[c][pt] = gf[c][pt] = 0.f;
        continue;
      }
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        cp_async4(&gu[c][pt], src[gc(c)] + g);
        if (w & kPtFirst) gf[c][pt] = 0.f;
        else cp_async4(&gf[c][pt], st.f[gc(c)] + g);
      }
    }
    cp_async_commit();
  };
  // asynchronous gather: the CTA's first work item is gathered here, each
  // later one while the CTA computes the item before it
  if (ASYNC && (int32_t)blockIdx.x < p.items()) {
    const int sv0 = p.locate(blockIdx.x);
    const DomainArgs &d = p.dom(sv0);
    const int pp0 = blockIdx.x - p.first(sv0);
    if (AXG_BOUND(d.patch_begin + pp0, d.n_patches, 1)) {
      const PatchMeta m0 = d.meta[d.patch_begin + pp0];
      if (threadIdx.x == 0) issue_words(d, 0, m0.pt_start, m0.n_pts);
      if (!mbar_wait_bounded(&s_wbar[0], 0u, p.state(sv0).err)) s_timeout = 1;
      issue_gather(p.state(sv0), 0, m0.n_pts);
    }
  }

  for (int32_t it = blockIdx.x; it < p.items(); it += gridDim.x) {
    if (it + (int32_t)gridDim.x >= p.items()) pdl_trigger();  // this CTA's last item: the next kernel may start
    // the work item's solve and patch
    const int sv = p.locate(it);
    const DomainArgs &d = p.dom(sv);
    const StateArgs &st = p.state(sv);
    const AnelArgs *an = ANEL ? p.anel(sv) : nullptr;
    const int pp = it - p.first(sv);
    // that solve has stopped (with the asynchronous gather, whose next item is
    // already in flight, a blown-up solve's items are computed on: its run
    // has failed either way)
    if (P::kMany && !ASYNC && __syncthreads_or(threadIdx.x == 0 && *st.blowup != 0)) continue;
    float stf1 = stf_one;
    if (TL && P::kMany && AXG_BOUND(*st.iter - 1, st.niter, 3)) stf1 = st.stf[*st.iter - 1];
    if (!AXG_BOUND(d.patch_begin + pp, d.n_patches, 1)) break;
    const PatchMeta m = d.meta[d.patch_begin + pp];
    const PatchRounds pr(m);
    const int buf = pcount % NB;
    float(*s_u)[ROW] = su_of(buf);
    float(*s_f)[ROW] = sf_of(buf);
    const uint32_t *s_w = sw_of(buf);
    // asynchronous gather: the next item's point words go to the other buffer now
    int next_npts = 0, next_sv = 0;
    if (ASYNC) {
      const int32_t itn = it + gridDim.x;
      if (itn < p.items()) {
        next_sv = p.locate(itn);
        const DomainArgs &dn = p.dom(next_sv);
        const int ppn = itn - p.first(next_sv);
        if (AXG_BOUND(dn.patch_begin + ppn, dn.n_patches, 1)) {
          const PatchMeta mn = dn.meta[dn.patch_begin + ppn];
          next_npts = mn.n_pts;
          if (threadIdx.x == 0) issue_words(dn, buf ^ 1, mn.pt_start, mn.n_pts);
        }
      }
    } else if (threadIdx.x == 0) {
      issue_words(d, 0, m.pt_start, m.n_pts);
    }
    // this warp's first STG element blocks
    WarpIter pf{0, warp};
    auto prefetch_first = [&]() {
      pf = WarpIter{0, warp};
      pf.norm(pr, warp);
      for (int q = 0; q < STG && pf.valid(pr); ++q) {
        if (lane == 0) {
          const int64_t el = (int64_t)m.elem_start + pf.s;
          if (AXG_BOUND(el, d.n_elem, 2)) issue(d, an, (kcount + q) % STG, el);
        }
        pf.s += kWarps;
        pf.norm(pr, warp);
      }
    };
    // 1. gather.  A point that an earlier writer (coupling pre-pass, earlier
    //    colour) already holds a partial sum for starts its accumulator from
    //    that sum, so that the write-back is a plain store.
    prefetch_first();
    if (ASYNC) {
      cp_async_wait_all();  // this thread's copies of the patch (issued during the previous one)
    } else {
      if (!mbar_wait_bounded(&s_wbar[0], pcount & 1u, st.err)) s_timeout = 1;
      // through registers: the compensated predictor or a symplectic drift on
      // the fly, or the stored predicted displacement (plain Newmark with
      // attenuation); kGB points per thread in flight cover a whole patch
      // (kGB * kThreads >= kMaxPatchPoints): one memory latency
      constexpr int kGB = (kMaxPatchPoints + kThreads - 1) / kThreads;
      for (int t0 = threadIdx.x; t0 < m.n_pts; t0 += kGB * kThreads) {
        uint32_t w[kGB];
        float uu[kGB][NC], ff[kGB][NC], cc[KAHAN ? kGB : 1][NC];
#pragma unroll
        for (int q = 0; q < kGB; ++q) {
          const int t = t0 + q * kThreads;
          w[q] = t < m.n_pts ? s_w[t] : kPtPad;
        }
#pragma unroll
        for (int q = 0; q < kGB; ++q) {
          const uint32_t g = w[q] & kPtIndexMask;
          const bool ok = w[q] != kPtPad && AXG_BOUND(g, st.nglob, 1);
          const bool part = ok && !(w[q] & kPtFirst);
#pragma unroll
          for (int c = 0; c < NC; ++c) {
            float u = ok ? (LOOK ? st.up[gc(c)][g] : st.u[gc(c)][g]) : 0.f;
            if (KAHAN) {
              float k = ok ? st.cu[gc(c)][g] : 0.f;
              // (a symplectic stage: hdt2 = 0, the compensated drift u + coefd(i) v)
              if (ok && MODE == MODE_SYMPLECTIC) u = drift_comp(u, st.v[gc(c)][g], st, k);
              else if (ok) u = predict_comp(u, st.v[gc(c)][g], st.a[gc(c)][g], st, k);
              cc[KAHAN ? q : 0][c] = k;
            } else if (ok && MODE == MODE_SYMPLECTIC) {
              u = u + mul2(st.dt, st.dt_lo, st.v[gc(c)][g]);  // drift: disp + velo * coefd(i)
            }  // (plain Newmark: up is the predicted displacement)
            uu[q][c] = u;
            ff[q][c] = part ? st.f[gc(c)][g] : 0.f;
          }
        }
#pragma unroll
        for (int q = 0; q < kGB; ++q) {
          const int t = t0 + q * kThreads;
          if (t < m.n_pts) {
#pragma unroll
            for (int c = 0; c < NC; ++c) {
              s_u[c][spos(t)] = uu[q][c];
              s_f[c][spos(t)] = ff[q][c];
              if (KAHAN) s_cu[c][spos(t)] = cc[KAHAN ? q : 0][c];
            }
          }
        }
      }
    }
    __syncthreads();

    // 2. elements, sub-round by sub-round
    int r0 = 0;
    for (int r = 0; r < pr.n; ++r) {
      const int r1 = pr.end(r);
      bool ready = r == 0;  // round r-1 complete (waited for)
      for (int s = r0 + warp; s < r1; s += kWarps) {
        int64_t el = (int64_t)m.elem_start + s;
        if (!AXG_BOUND(el, d.n_elem, 2)) el = 0;
        const uint32_t slot = kcount % STG;
        if (!mbar_wait_bounded(&my_bars[slot], (kcount / STG) & 1u, st.err)) s_timeout = 1;
        const float *blk = my_ring + slot * BS;
        const int32_t info = *reinterpret_cast<const int32_t *>(blk + solid_info_off(NT));
        int axslot = (info & 0xFFFFFF) - 1;
        if (axslot >= 0 && !AXG_BOUND((int64_t)(axslot + 1) * NA * 5 - 1, d.n_m0, 2)) axslot = -1;
        int idx = active ? reinterpret_cast<const uint16_t *>(blk + solid_idx_off(NT))[lane] : 0;
        if (!AXG_BOUND(idx, m.n_pts, 2)) idx = 0;
        idx = spos(idx);
        float u[3] = {0.f, 0.f, 0.f};
        if (active) {
          u[0] = s_u[0][idx];
          if (POLE == POLE_MONO) {
            u[2] = s_u[1][idx];
          } else {
            u[1] = s_u[1][idx];
            u[2] = s_u[2][idx];
          }
        }
        if (TL && lane == 6) {
          // runtime_info guard on disp(1,1,:,:) (SOLVER/time_evol_wave.F90:1042)
          const float mx = fmaxf(fabsf(u[0]), fmaxf(fabsf(u[1]), fabsf(u[2])));
          if (!(mx <= st.thresh)) atomicCAS(st.blowup, 0, *st.iter);
        }
        const bool ax = axslot >= 0;
        if (ax && i == 0) {  // apply_axis_mask_{one,two,three}comp on disp
          if (POLE == POLE_MONO) u[0] = 0.f;
          if (POLE == POLE_DI) { u[1] = 0.f; u[2] = 0.f; }
          if (POLE == POLE_QUAD) { u[0] = 0.f; u[1] = 0.f; u[2] = 0.f; }
        }
        float f0, f1 = 0.f, f2;
        float gx[3], ge[3];
        const float *m0 = ax ? d.m0 + (int64_t)axslot * (NA * 5) : nullptr;
        if (POLE == POLE_MONO) {
          if (ax) stiff_mono<true>(coef, blk, m0, ml, i, j, u[0], u[2], f0, f2, gx, ge);
          else stiff_mono<false>(coef, blk, m0, ml, i, j, u[0], u[2], f0, f2, gx, ge);
        } else if (POLE == POLE_DI) {
          if (ax) stiff_di<true>(coef, blk, m0, ml, i, j, u[0], u[1], u[2], f0, f1, f2, gx, ge);
          else stiff_di<false>(coef, blk, m0, ml, i, j, u[0], u[1], u[2], f0, f1, f2, gx, ge);
        } else {
          if (ax) stiff_quad<true>(coef, blk, m0, ml, i, j, u[0], u[1], u[2], f0, f1, f2, gx, ge);
          else stiff_quad<false>(coef, blk, m0, ml, i, j, u[0], u[1], u[2], f0, f1, f2, gx, ge);
        }
        float *ablk = my_aring + slot * AS;  // attenuation constants, then state
        if (ANEL) {
          // A Newmark step updates the memory variables here, from the
          // predicted, masked displacement (time_step_memvars after
          // pdistsum_solid in SOLVER/time_evol_wave.F90), and the anelastic
          // stiffness takes their sum from before the update, as the
          // reference's acc1 does.  (A symplectic stage only reads them:
          // anel_memvar_kernel updates them once per step.)
          const float rs =
              MODE == MODE_NEWMARK
                  ? anel_memvar_step<POLE>(ablk, ablk + kAnelConst, scr + warp * 32, *an, cg, kcg, lane, u, gx, ge)
                  : memvar_sum(ablk + kAnelConst, an->nsls, lane);
          if (ax) anel_stiffness<POLE, true>(coef, ablk, rs, cg, kcg, i, j, active, lane, f0, f1, f2);
          else anel_stiffness<POLE, false>(coef, ablk, rs, cg, kcg, i, j, active, lane, f0, f1, f2);
        }
        if (MODE == MODE_NEWMARK && !ANEL && d.fx && active) {
          // attenuation at every GLL point: minus the anelastic stiffness
          // (glob_anel_stiffness_*_4), formed by anel_full_kernel
          const float *x = d.fx + el * 75;
          f0 = f0 + x[lane];
          f1 = f1 + x[25 + lane];
          f2 = f2 + x[50 + lane];
        }
        if (ax && i == 0) {  // axis mask of acc1
          if (POLE == POLE_MONO) f0 = 0.f;
          if (POLE == POLE_DI) { f1 = 0.f; f2 = 0.f; }
          if (POLE == POLE_QUAD) { f0 = 0.f; f1 = 0.f; f2 = 0.f; }
        }
        // the previous sub-round's accumulations must be complete; the wait
        // comes after this element's stiffness, which hides it
        if (!ready) {
          if (!mbar_wait_bounded(&s_round[r - 1], (round_par >> (r - 1)) & 1u, st.err)) s_timeout = 1;
          ready = true;
        }
        if (active) {
          s_f[0][idx] += f0;
          if (POLE == POLE_MONO) {
            s_f[1][idx] += f2;
          } else {
            s_f[1][idx] += f1;
            s_f[2][idx] += f2;
          }
        }
        if (ANEL && MODE == MODE_NEWMARK) {
          // the element's updated state back to HBM
          __syncwarp();
          const float4 *src4 = reinterpret_cast<const float4 *>(ablk + kAnelConst);
          float4 *dst4 = reinterpret_cast<float4 *>(an->state + el * an->state_stride);
          for (int q = lane; q < an->state_stride / 4; q += 32) dst4[q] = src4[q];
        }
        // the slot is free again: start the copy of the element STG ahead
        __syncwarp();
        if (pf.valid(pr)) {
          if (lane == 0) {
            const int64_t pel = (int64_t)m.elem_start + pf.s;
            fence_proxy_async();  // the warp's reads of the slot precede the async-proxy write
            if (AXG_BOUND(pel, d.n_elem, 2)) issue(d, an, slot, pel);
          }
          pf.s += kWarps;
          pf.norm(pr, warp);
        }
        ++kcount;
      }
      mbar_arrive(&s_round[r]);  // this thread's accumulations of round r are done
      r0 = r1;
      if (ASYNC && r == 0 && next_npts > 0) {
        // the next item's words have landed in the other buffer: start its gather
        if (!mbar_wait_bounded(&s_wbar[buf ^ 1], ((pcount + 1) / NB) & 1u, st.err)) s_timeout = 1;
        issue_gather(p.state(next_sv), buf ^ 1, next_npts);
      }
    }
    round_par ^= (1u << pr.n) - 1u;  // each used s_round completed once in this patch
    __syncthreads();

    // 3. write-back
    if (MODE == MODE_FORCE) {
      for (int t = threadIdx.x; t < m.n_pts; t += kThreads) {
        const uint32_t g = s_w[t] & kPtIndexMask;
        if (!AXG_BOUND(g, st.nglob, 3)) continue;
#pragma unroll
        for (int c = 0; c < NC; ++c) st.f[gc(c)][g] = s_f[c][spos(t)];
      }
    } else {
      // kWB points per thread at a time: all of their loads (velocity,
      // acceleration, inverse mass, gamma) are issued before any store, so
      // that one memory latency covers them (stores to the same arrays would
      // otherwise keep the compiler from hoisting the next point's loads)
      constexpr int kWB = 3;
      for (int t0 = threadIdx.x; t0 < m.n_pts; t0 += kWB * kThreads) {
        uint32_t w[kWB];
        float vel[kWB][NC], acc[kWB][NC], im[kWB], gam[kWB], kv[KAHAN ? kWB : 1][NC];
        double imd[KAHAN ? kWB : 1];  // compensated mode: the FP64 inverse mass, when the handle has it
#pragma unroll
        for (int q = 0; q < kWB; ++q) {
          const int t = t0 + q * kThreads;
          w[q] = t < m.n_pts ? s_w[t] : kPtPad;
          const uint32_t g = w[q] & kPtIndexMask;
          const bool last = w[q] != kPtPad && (w[q] & kPtLast) && AXG_BOUND(g, st.nglob, 3);
          im[q] = last ? st.inv_mass[g] : 0.f;
          if (KAHAN) imd[KAHAN ? q : 0] = last && st.inv_mass_dp ? st.inv_mass_dp[g] : 0.0;
          gam[q] = last && st.gamma ? st.gamma[g] : 0.f;
#pragma unroll
          for (int c = 0; c < NC; ++c) {
            vel[q][c] = last ? st.v[gc(c)][g] : 0.f;
            acc[q][c] = last && MODE == MODE_NEWMARK ? st.a[gc(c)][g] : 0.f;
            if (KAHAN) kv[KAHAN ? q : 0][c] = last ? st.cv[gc(c)][g] : 0.f;
          }
        }
#pragma unroll
        for (int q = 0; q < kWB; ++q) {
          const int t = t0 + q * kThreads;
          if (w[q] == kPtPad) continue;
          const uint32_t g = w[q] & kPtIndexMask;
          if (!AXG_BOUND(g, st.nglob, 3)) continue;
          float v[NC];
#pragma unroll
          for (int c = 0; c < NC; ++c) v[c] = s_f[c][spos(t)];
          if (!(w[q] & kPtLast)) {
#pragma unroll
            for (int c = 0; c < NC; ++c) st.f[gc(c)][g] = v[c];
            continue;
          }
          // last writer: source, corrector, store the new state
          if ((w[q] & kPtSource) && stf1 != 0.f) {
            for (int k = 0; k < st.src.n; ++k)
              if ((uint32_t)st.src.gidx[k] == g) {
                if (KAHAN && st.src.val_dp) {  // the source projection in FP64, one rounding
#pragma unroll
                  for (int c = 0; c < NC; ++c)
                    v[c] = (float)((double)v[c] - st.src.val_dp[3 * k + gc(c)] * (double)stf1);
                } else {
#pragma unroll
                  for (int c = 0; c < NC; ++c) v[c] = v[c] - st.src.val[3 * k + gc(c)] * stf1;
                }
              }
          }
#pragma unroll
          for (int c = 0; c < NC; ++c) {
            const int cg = gc(c);
            const float dsp = s_u[c][spos(t)];
            if (MODE == MODE_SYMPLECTIC) {
              // kick (SOLVER/time_evol_wave.F90:688-717): acc = -inv_mass acc
              // [- absorbing terms], velo += acc * coefv(i); the dipole's z
              // component takes twice the whole acceleration
              float a = (KAHAN && st.inv_mass_dp) ? (float)(-imd[KAHAN ? q : 0] * (double)v[c]) : -im[q] * v[c];
              if (st.gamma) a = a - 2.f * gam[q] * vel[q][c] - gam[q] * gam[q] * dsp;
              const bool two = POLE == POLE_DI && cg == 2;
              const float dv = mul2(two ? 2.f * st.kick : st.kick, two ? 2.f * st.kick_lo : st.kick_lo, a);
              if (KAHAN) {
                float k = kv[KAHAN ? q : 0][c];
                st.v[cg][g] = kahan_add(vel[q][c], dv, k);
                st.cv[cg][g] = k;
                st.cu[cg][g] = s_cu[c][spos(t)];
              } else {
                st.v[cg][g] = vel[q][c] + dv;
              }
              st.a[cg][g] = a;
              const bool zero = (w[q] & kPtAxis) && axis_masked<POLE>(cg);
              st.u[cg][g] = zero ? 0.f : dsp;
              if (KAHAN && zero) st.cu[cg][g] = 0.f;
              continue;
            }
            float a;
            if (KAHAN && st.inv_mass_dp) {  // the inverse mass in FP64, one rounding
              const double md = imd[KAHAN ? q : 0];
              a = (float)((POLE == POLE_DI && cg == 2) ? (-2.0 * md) * (double)v[c] : -md * (double)v[c]);
            } else {
              a = (POLE == POLE_DI && cg == 2) ? (-2.f * im[q]) * v[c] : -im[q] * v[c];
            }
            if (st.gamma) a = a - 2.f * gam[q] * vel[q][c] - gam[q] * gam[q] * dsp;
            float vn;
            if (KAHAN) {
              float k = kv[KAHAN ? q : 0][c];
              vn = kahan_add(vel[q][c], mul2(st.hdt, st.hdt_lo, acc[q][c] + a), k);
              st.cv[cg][g] = k;
              st.cu[cg][g] = comp_after_step(s_cu[c][spos(t)], vn, a, st);
            } else {
              vn = vel[q][c] + mul2(st.hdt, st.hdt_lo, acc[q][c] + a);
            }
            st.v[cg][g] = vn;
            st.a[cg][g] = a;
            // the axis masks of the reference zero these components of its state
            const bool zero = (w[q] & kPtAxis) && axis_masked<POLE>(cg);
            const float un = zero ? 0.f : dsp;
            if (LOOK) {
              // The new displacement is the gathered prediction, which stays
              // in the buffer it came from (up, with the masked components of
              // axis points stored as zero): st.u is the other buffer, and
              // receives the next step's predictor disp + deltat*velo +
              // half_dt_sq*acc0 (SOLVER/time_evol_wave.F90:357-364).
              st.u[cg][g] = zero ? 0.f : predict(un, vn, a, st);
            } else {
              st.u[cg][g] = un;
            }
            if (KAHAN && zero) st.cu[cg][g] = 0.f;
          }
        }
      }
    }
    __syncthreads();
    ++pcount;
  }
  // After a timeout, bulk copies of this CTA may still be in flight into its
  // shared memory: wait (bounded) for the last phase of each ring slot and of
  // the point-word buffer before the CTA exits.
  __syncthreads();
  if (s_timeout) {
    if (lane == 0)
      for (uint32_t q = 0; q < (uint32_t)STG && q < kcount; ++q) {
        const uint32_t k = kcount - 1 - q;  // the last element consumed from slot k % STG
        mbar_drain(&my_bars[k % STG], (k / STG) & 1u);
      }
    if (threadIdx.x == 0 && pcount > 0) {
      const uint32_t b = ASYNC ? (pcount - 1) % NB : 0u;
      const uint32_t par = ASYNC ? ((pcount - 1) / NB) & 1u : (pcount - 1) & 1u;
      mbar_drain(&s_wbar[b], par);
    }
  }
}

// ------------------------------------------------------------ attenuation at every GLL point
//
// att_coarse_grained = .false.: memory variables at all 25 GLL points of
// every solid element.  Per launch slot the host packs kFullConst constants:
// [field][GLL point] of delta_mu, delta_kappa, Y, V_s_eta, V_s_xi, V_z_eta,
// V_z_xi, DsDeta_over_J_sol, DzDeta_over_J_sol, DsDxi_over_J_sol,
// DzDxi_over_J_sol, inv_s_solid; then [field][jpol] of Y0, V0_s_eta,
// V0_s_xi, V0_z_eta, V0_z_xi (zero off the axis); then the two Q-table rows.
// The state of a slot is memory_var(0:4,0:4,6,n_sls), src_tr_tm1(0:4,0:4),
// src_dev_tm1(0:4,0:4,6), the reference's layouts.
enum : int {
  F_DMU = 0, F_DKA = 25, F_Y = 50, F_VSE = 75, F_VSX = 100, F_VZE = 125, F_VZX = 150, F_DSDETA = 175,
  F_DZDETA = 200, F_DSDXI = 225, F_DZDXI = 250, F_INVS = 275, F_Y0 = 300, F_V0SE = 305, F_V0SX = 310,
  F_V0ZE = 315, F_V0ZX = 320, F_QMU = 325, F_QKA = 326
};
constexpr int kFullConst = 328;  // floats, a 16-byte multiple
__host__ __device__ constexpr int full_state_stride(int nsls) { return ((150 * nsls + 175 + 3) / 4) * 4; }

struct FullAnelArgs {
  AnelArgs an;            // consts (kFullConst per slot), state, qtab, ex, nsls, state_stride, n_q
  float *fx;              // per slot 3 x 25: minus the anelastic stiffness the next Newmark step adds
  const int32_t *gidx;    // per slot the element's 25 global points
  const uint8_t *axial;   // per slot 1 for an axial element
  int64_t nel;
};

// One warp per element (launch order), lane = GLL point.  UPDATE: the memory
// variables of the step from the displacement the step stored
// (time_step_memvars_4 with compute_strain_att_el_4, SOLVER/attenuation.f90:
// 210-334, 542-606: the gradients of axisym_gradient_solid_el_4, f / s of
// f_over_s_solid_el_4 with L'Hospital's df/ds on the axis).  Then, from the
// memory variables, the anelastic stiffness of glob_anel_stiffness_*_4
// (SOLVER/stiffness_mono.f90:409-507, SOLVER/stiffness_di.f90:604-723,
// SOLVER/stiffness_quad.f90:555-669), stored negated in fx for the next
// step's patch kernel.  Without UPDATE (before a run) only the latter.
template <int POLE, bool UPDATE>
__global__ void __launch_bounds__(kThreads) anel_full_kernel(const __grid_constant__ FullAnelArgs fa, StateArgs st,
                                                             SpecDev sp) {
  pdl_wait();
  pdl_trigger();
  if (*st.blowup) return;
  const AnelArgs &an = fa.an;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool active = lane < 25;
  const int ml = active ? lane : 24;
  const int i = ml % 5, j = ml / 5, j5 = 5 * j;
  LaneCoef coef;
  load_coef(sp, i, j, coef);
  const int nsls = an.nsls;
  for (int64_t el = (int64_t)blockIdx.x * kWarps + warp; el < fa.nel; el += (int64_t)gridDim.x * kWarps) {
    const float *cs = an.consts + el * kFullConst;
    float *R = an.state + el * an.state_stride;
    float *trm1 = R + 150 * nsls, *devm1 = trm1 + 25;
    const bool ax = fa.axial[el] != 0;
    if (UPDATE) {
      int32_t g = fa.gidx[25 * el + ml];
      if (!AXG_BOUND(g, st.nglob, 52)) g = 0;
      float u[3] = {st.u[0][g], POLE == POLE_MONO ? 0.f : st.u[1][g], st.u[2][g]};
      if (ax && i == 0) {  // apply_axis_mask_* on disp
        if (POLE == POLE_MONO) u[0] = 0.f;
        if (POLE == POLE_DI) { u[1] = 0.f; u[2] = 0.f; }
        if (POLE == POLE_QUAD) { u[0] = 0.f; u[1] = 0.f; u[2] = 0.f; }
      }
      const float dsdeta = cs[F_DSDETA + ml], dzdeta = cs[F_DZDETA + ml];
      const float dsdxi = cs[F_DSDXI + ml], dzdxi = cs[F_DZDXI + ml], invs = cs[F_INVS + ml];
      // axisym_gradient_solid_el_4 of the field f held lane-wise: (d/ds, d/dz)
      auto grad = [&](float f, float &gs, float &gz) {
        const float m1 = ax ? dxi(f, coef.xi1, j5) : dxi(f, coef.xi2, j5);
        const float m2 = deta(f, coef.eta, i);
        gs = dzdeta * m1 + dzdxi * m2;
        gz = dsdeta * m1 + dsdxi * m2;
      };
      // f_over_s_solid_el_4: f / s; on the axis (ipol = 0 of an axial
      // element) df/ds (dsdf_elem_solid, G1T); the contractions run on every
      // lane of the warp (ax is uniform across it)
      auto fos = [&](float f) {
        float o = invs * f;
        if (ax) {
          float gs, gz;
          grad(f, gs, gz);
          if (i == 0) o = gs;
        }
        return o;
      };
      float gu[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // Voigt 1..6
      float b1s, b1z, b2s, b2z;
      grad(POLE == POLE_DI ? u[0] + u[1] : u[0], b1s, b1z);
      grad(u[2], b2s, b2z);
      gu[0] = b1s;
      gu[2] = b2z;
      gu[4] = b1z + b2s;
      if (POLE == POLE_MONO) {
        gu[1] = fos(u[0]);
      } else if (POLE == POLE_DI) {
        gu[1] = 2.f * fos(u[1]);
        grad(u[0] - u[1], b1s, b1z);
        const float t = fos(u[2]);
        gu[3] = -t - b1z;
        gu[5] = -gu[1] - b1s;
      } else {
        gu[1] = fos(u[0] - 2.f * u[1]);
        grad(u[1], b1s, b1z);
        const float t = fos(u[2]);
        const float t2 = fos(u[1] - 2.f * u[0]);
        gu[3] = -2.f * t - b1z;
        gu[5] = t2 - b1s;
      }
      if (active) {
        const float tr = gu[0] + gu[1] + gu[2];
        const float dm = cs[F_DMU + lane], dk = cs[F_DKA + lane];
        float src_dev[6];
#pragma unroll
        for (int v = 0; v < 3; ++v) src_dev[v] = (dm * 2.f) * (gu[v] - tr * (1.f / 3.f));
        src_dev[3] = POLE == POLE_MONO ? 0.f : dm * gu[3];
        src_dev[4] = dm * gu[4];
        src_dev[5] = POLE == POLE_MONO ? 0.f : dm * gu[5];
        const float src_tr = dk * tr;
        int qmu = __float_as_int(cs[F_QMU]), qka = __float_as_int(cs[F_QKA]);
        if (!AXG_BOUND(qmu, an.n_q, 52)) qmu = 0;
        if (!AXG_BOUND(qka, an.n_q, 52)) qka = 0;
        const float *tmu = an.qtab + qmu * 2 * kMaxSls, *tka = an.qtab + qka * 2 * kMaxSls;
        const float trp = trm1[lane];
        for (int q = 0; q < nsls; ++q) {
          const float trb = __ldg(tka + q) * src_tr + __ldg(tka + kMaxSls + q) * trp;
#pragma unroll
          for (int v = 0; v < 6; ++v) {
            if (POLE == POLE_MONO && (v == 3 || v == 5)) continue;  // never written for the monopole
            float *r = R + lane + 25 * (v + 6 * q);
            const float db = __ldg(tmu + q) * src_dev[v] + __ldg(tmu + kMaxSls + q) * devm1[lane + 25 * v];
            float nv = an.ex[q] * *r + db;
            if (v < 3) nv = nv + trb;
            *r = nv;
          }
        }
        trm1[lane] = src_tr;
#pragma unroll
        for (int v = 0; v < 6; ++v) devm1[lane + 25 * v] = src_dev[v];
      }
      __syncwarp();
    }
    // the summed memory variables at the lane's point
    float r[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (active)
      for (int q = 0; q < nsls; ++q)
#pragma unroll
        for (int v = 0; v < 6; ++v) r[v] = r[v] + R[lane + 25 * (v + 6 * q)];
    const float yl = cs[F_Y + ml], vse = cs[F_VSE + ml], vsx = cs[F_VSX + ml];
    const float vze = cs[F_VZE + ml], vzx = cs[F_VZX + ml];
    // X = mxm(G, S) (G1 on axial elements) and mxm(S, G2T)
    auto gx = [&](float S) { return ax ? dxi(S, coef.sxi1, j5) : dxi(S, coef.sxi2, j5); };
    auto ge = [&](float S) { return deta(S, coef.seta, i); };
    // axial vectors at jpol = j (lanes with ipol = 0 use them)
    const float y0 = cs[F_Y0 + j], v0se = cs[F_V0SE + j], v0sx = cs[F_V0SX + j];
    const float v0ze = cs[F_V0ZE + j], v0zx = cs[F_V0ZX + j];
    // outerprod(G0, V)(i, j) = G0(i) V(j), V held by lane (0, j)
    auto outer = [&](float V) { return coef.g0i * __shfl_sync(kFull, V, j5); };
    float l0, l1 = 0.f, l2;
    if (POLE == POLE_MONO) {
      const float S1s = vze * r[0] + vse * r[4], S2s = vzx * r[0] + vsx * r[4];
      const float S1z = vze * r[4] + vse * r[2], S2z = vzx * r[4] + vsx * r[2];
      l0 = gx(S1s) + ge(S2s) + yl * r[1];
      l2 = gx(S1z) + ge(S2z);
      if (ax) {
        const float V1 = v0ze * r[0] + v0se * r[4] + y0 * r[1];
        const float V2 = v0ze * r[4] + v0se * r[2];
        const float V3 = v0zx * r[4] + v0sx * r[2];
        const float V4 = deta(V3, coef.seta, 0);  // vxm(V3, G2T) on the lanes with ipol = 0
        l0 = l0 + outer(V1);
        l2 = l2 + outer(V2);
        if (i == 0) l2 = l2 + V4;
      }
    } else if (POLE == POLE_DI) {
      const float r16m = r[0] - r[5], r54m = r[4] - r[3], r16p = r[0] + r[5], r54p = r[4] + r[3];
      const float S1p = vze * r16m + vse * r54m, S2p = vzx * r16m + vsx * r54m;
      const float S1m = vze * r16p + vse * r54p, S2m = vzx * r16p + vsx * r54p;
      const float S1z = vze * r[4] + vse * r[2], S2z = vzx * r[4] + vsx * r[2];
      l0 = gx(S1p) + ge(S2p);
      l1 = gx(S1m) + ge(S2m) + 2.f * yl * (r[1] - r[5]);
      l2 = gx(S1z) + ge(S2z) - yl * r[3];
      if (ax) {
        const float V1 = v0ze * r16m + v0se * r54m;
        const float V2 = v0zx * r16m + v0sx * r54m;
        const float V3 = deta(V2, coef.seta, 0);
        l0 = l0 + outer(V1);
        if (i == 0) l0 = l0 + V3;
        const float V1m = v0ze * r16p + v0se * r54p + y0 * 2.f * (r[1] - r[5]);
        l1 = l1 + outer(V1m);
        l2 = l2 + outer(V2);  // the reference adds V2 here, as it writes it
      }
    } else {
      const float S1s = vze * r[0] + vse * r[4], S2s = vzx * r[0] + vsx * r[4];
      const float S1p = vze * r[5] + vse * r[3], S2p = vzx * r[5] + vsx * r[3];
      const float S1z = vze * r[4] + vse * r[2], S2z = vzx * r[4] + vsx * r[2];
      l0 = gx(S1s) + ge(S2s) + yl * (r[1] - 2.f * r[5]);
      l1 = -gx(S1p) - ge(S2p) + yl * (r[5] - 2.f * r[1]);
      l2 = gx(S1z) + ge(S2z) - 2.f * yl * r[3];
      if (ax) {
        l0 = l0 + outer(v0ze * r[0] + y0 * (r[1] - 2.f * r[5]));
        l1 = l1 + outer(-v0ze * r[5] + y0 * (r[5] - 2.f * r[1]));
        l2 = l2 + outer(v0se * r[2]);
      }
    }
    if (active) {
      float *x = fa.fx + el * 75;
      x[lane] = -l0;
      x[25 + lane] = -l1;
      x[50 + lane] = -l2;
    }
    __syncwarp();
  }
}

// time_step_memvars (SOLVER/attenuation.f90:81-202) once per step of the
// symplectic loop, after the final drift (SOLVER/time_evol_wave.F90:727-731):
// one warp per element in launch order (the order of the attenuation data),
// the masked displacement gathered from its points, the first-stage
// derivatives as in the stiffness (G1T on axial elements), then the same
// update as the Newmark kernel's, on the state in HBM.
template <int POLE>
__global__ void __launch_bounds__(kThreads) anel_memvar_kernel(const __grid_constant__ AnelArgs an,
                                                               const int32_t *gidx, const uint8_t *axial,
                                                               StateArgs st, int64_t nel, SpecDev sp) {
  __shared__ float scr_all[kWarps * 32];
  if (*st.blowup) return;  // no block-wide synchronisation below
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool active = lane < 25;
  const int ml = active ? lane : 24;
  const int i = ml % 5, j = ml / 5, j5 = 5 * j;
  LaneCoef coef;
  load_coef(sp, i, j, coef);
  const bool cg = active && (i == 1 || i == 3) && (j == 1 || j == 3);
  const int kcg = 2 * (i >> 1) + (j >> 1);
  float *scr = scr_all + warp * 32;
  for (int64_t el = (int64_t)blockIdx.x * kWarps + warp; el < nel; el += (int64_t)gridDim.x * kWarps) {
    int32_t g = gidx[25 * el + ml];
    if (!AXG_BOUND(g, st.nglob, 51)) g = 0;
    const bool ax = axial[el] != 0;
    float u[3] = {st.u[0][g], POLE == POLE_MONO ? 0.f : st.u[1][g], st.u[2][g]};
    if (ax && i == 0) {  // apply_axis_mask_* on disp
      if (POLE == POLE_MONO) u[0] = 0.f;
      if (POLE == POLE_DI) { u[1] = 0.f; u[2] = 0.f; }
      if (POLE == POLE_QUAD) { u[0] = 0.f; u[1] = 0.f; u[2] = 0.f; }
    }
    float gx[3], ge[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      gx[c] = ax ? dxi(u[c], coef.xi1, j5) : dxi(u[c], coef.xi2, j5);
      ge[c] = deta(u[c], coef.eta, i);
    }
    anel_memvar_step<POLE>(an.consts + el * kAnelConst, an.state + el * an.state_stride, scr, an, cg, kcg, lane, u,
                           gx, ge);
    __syncwarp();
  }
}

// One solve: the patches of one colour.  The arguments are plain by-value
// parameters, so that the body reads them as constant-bank operands.
template <int POLE, int MODE, bool ANEL, bool KAHAN>
__global__ void __launch_bounds__(kThreads, solid_min_ctas(MODE, ANEL, KAHAN))
    solid_patch_kernel(DomainArgs d, StateArgs st, SpecDev sp, int32_t n_colour_patches,
                       const __grid_constant__ AnelArgs an) {  // an.ex[] is indexed at run time
  solid_patch_body<POLE, MODE, ANEL, KAHAN>(OneSolve{d, st, n_colour_patches, an}, sp);
}

// A batch: colour c of every solve of the launch (a Newmark step, or one
// stage of a symplectic step), found by run-time index into the descriptors
// (hence in the parameter space, __grid_constant__).
template <int POLE, int MODE, bool KAHAN>
__global__ void __launch_bounds__(kThreads, solid_min_ctas(MODE, false, KAHAN))
    solid_batch_kernel(const __grid_constant__ Many<PatchWork> p, SpecDev sp) {
  solid_patch_body<POLE, MODE, false, KAHAN>(ManySolves{p, nullptr}, sp);
}
// An attenuated batch: the same, with each solve's attenuation data (cg4)
// beside its descriptors.
template <int POLE, int MODE, bool KAHAN>
__global__ void __launch_bounds__(kThreads, solid_min_ctas(MODE, true, KAHAN))
    solid_anel_batch_kernel(const __grid_constant__ Many<PatchWork> p, SpecDev sp,
                            const __grid_constant__ AnelBatch an) {
  solid_patch_body<POLE, MODE, true, KAHAN>(ManySolves{p, an.a}, sp);
}

// ------------------------------------------------------------ fluid kernels
//
// The fluid step runs in two fully parallel passes instead of coloured
// patches: the element pass computes every element's stiffness contribution
// (glob_fluid_stiffness_4 with its source and masks) into a per-element
// buffer, the point pass sums each global point's contributions in a fixed
// order (the CSR of its (element, GLL point) copies: pdistsum_fluid) after
// the coupling pre-pass's partial sum, and applies the corrector.  Both are
// plain streams over HBM with no barriers, so the fluid's small element work
// is no longer bound by the latency of patch-sized phases.

// The element arrays of the fluid (points, metric terms, free-surface mask,
// contributions) are stored in chunks of kFlChunk element slots: value v of
// slot e at fl_at(e, v, nv) for nv values per element, the chunk's 32
// elements side by side, so that a warp of 32 consecutive elements loads or
// stores one value as one 128-byte line.
constexpr int kFlChunk = 32;
__host__ __device__ constexpr int64_t fl_chunks(int64_t nel) { return (nel + kFlChunk - 1) / kFlChunk; }
__host__ __device__ constexpr int64_t fl_at(int64_t e, int v, int nv) {
  return (e / kFlChunk) * ((int64_t)nv * kFlChunk) + (int64_t)v * kFlChunk + (e % kFlChunk);
}

struct FluidArgs {
  const int32_t *gidx;     // chunked, 25 values per element slot (launch order): its global points
  const float *metric;     // chunked, 25 nt values per slot: M1chi, M2chi, M4chi [, M_w_fl] at 25 t + p
  const int32_t *elinfo;   // per element slot: bits 0..23 axial slot + 1, bits 24..27 source slot + 1
  const float *m0;         // per axial slot 5 floats (M0_w_fl)
  const float *fsmask;     // chunked, 25 values per slot (fluid free-surface mask) or null
  const float *srcfl;      // fluid source terms (8, 25) or null
  const int32_t *start;    // nglob + 1: each point's first copy in ent; bit 31 of start[g]: the point
                           // holds a coupling pre-pass partial sum (in the force array); bit 30: on the axis
  const int32_t *ent;      // 25 nel: the fel index of each copy, points in order
  float *fel;              // chunked, 25 values per slot: the element contributions of the step
  int64_t nel, nglob, n_m0;  // extents (checked builds)
};
constexpr uint32_t kFlPartial = 1u << 31, kFlAxis = 1u << 30, kFlStartMask = kFlAxis - 1u;

struct FluidWork {
  FluidArgs fa;
  StateArgs st;
};

// chi at the step's gather point: the plain Newmark step's stored prediction,
// the compensated predictor, a symplectic stage's drift (compensated or not)
template <int MODE, bool KAHAN>
__device__ __forceinline__ float fluid_predicted(const StateArgs &st, int64_t g, float &k) {
  if (KAHAN) {
    k = st.cu[0][g];
    if (MODE == MODE_SYMPLECTIC) return drift_comp(st.u[0][g], st.v[0][g], st, k);
    return predict_comp(st.u[0][g], st.v[0][g], st.a[0][g], st, k);
  }
  if (MODE == MODE_SYMPLECTIC) return st.u[0][g] + mul2(st.dt, st.dt_lo, st.v[0][g]);  // chi + dchi * coefd(i)
  return st.up[0][g];
}

// glob_fluid_stiffness_4 (SOLVER/stiffness_fluid.f90:139-216) of one element
// held by one thread: chi(i, j) at chi[i + 5 j] in, the element's
// contributions out.  met points at the element's first metric value (value
// v at met[v * kFlChunk]).  The products and summation order of the shuffle
// contractions dxi / deta: first stage X1 = mxm_4(G2T or G1T, chi),
// X2 = mxm_4(chi, G2); S1 = M1chi X2 + M2chi X1, S2 = M1chi X1 + M4chi X2;
// second stage mxm_4(G2 or G1, S1) + mxm_4(S2, G2T); for the non-monopole
// sources + M_w_fl chi and, on the axis, G0(i) M0_w_fl(j) mxm_4(G0, chi).
template <bool AX, bool NONMONO>
__device__ __forceinline__ void fluid_elem_stiffness(const SpecDev &sp, const float *met, const float *m0,
                                                     const float (&chi)[25], float (&loc)[25]) {
  // G(a, b) of the xi direction: G1 on axial elements
  auto gx = [&](int a, int b) { return AX ? sp.g1[a + 5 * b] : sp.g2[a + 5 * b]; };
  float S1[25], S2[25];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const int q = i + 5 * j;
      float x1 = gx(0, i) * chi[5 * j];
#pragma unroll
      for (int k = 1; k < 5; ++k) x1 = fmaf(gx(k, i), chi[k + 5 * j], x1);
      float x2 = chi[i] * sp.g2[5 * j];
#pragma unroll
      for (int k = 1; k < 5; ++k) x2 = fmaf(chi[i + 5 * k], sp.g2[k + 5 * j], x2);
      const float m1 = __ldg(met + q * kFlChunk), m2 = __ldg(met + (25 + q) * kFlChunk),
                  m4 = __ldg(met + (50 + q) * kFlChunk);
      S1[q] = m1 * x2 + m2 * x1;
      S2[q] = m1 * x1 + m4 * x2;
    }
  }
#pragma unroll
  for (int j = 0; j < 5; ++j) {
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const int q = i + 5 * j;
      float y1 = gx(i, 0) * S1[5 * j];
#pragma unroll
      for (int k = 1; k < 5; ++k) y1 = fmaf(gx(i, k), S1[k + 5 * j], y1);
      float y2 = S2[i] * sp.g2[j];
#pragma unroll
      for (int k = 1; k < 5; ++k) y2 = fmaf(S2[i + 5 * k], sp.g2[j + 5 * k], y2);
      float l = y1 + y2;
      if (NONMONO) {
        l = l + __ldg(met + (75 + q) * kFlChunk) * chi[q];
        if (AX) {
          float v1 = sp.g0[0] * chi[5 * j];
#pragma unroll
          for (int k = 1; k < 5; ++k) v1 = fmaf(sp.g0[k], chi[k + 5 * j], v1);
          l = l + sp.g0[i] * (m0[j] * v1);
        }
      }
      loc[q] = l;
    }
  }
}

// Element pass: one thread per element (items: the elements of the solves).
// The thread gathers its 25 points' chi with the predictor, computes the
// element's stiffness with its source, axial mask and free-surface mask in
// registers, and stores its 25 contributions.  The element's 25 gathers and
// its metric loads are independent of one another, so each thread has tens
// of loads in flight, and there are no shuffles.
// CTAs of 128 threads, five per SM at 96 registers (20 warps; 256-thread
// CTAs at 128 registers held 16)
constexpr int kFlElemThreads = 128;
template <int NONMONO, int MODE, bool KAHAN, class P = One<FluidWork>>
__global__ void __launch_bounds__(kFlElemThreads, 5) fluid_elem_kernel(const __grid_constant__ P p, SpecDev sp) {
  pdl_wait();
  pdl_trigger();
  const int32_t it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= p.items()) return;
  const int sv = p.locate(it);
  const FluidArgs &f = p.at(sv).fa;
  const StateArgs &st = p.at(sv).st;
  if (*st.blowup) return;  // (a stopped solve of a batch: its contributions are not used)
  const int64_t el = it - p.first(sv);
  if (!AXG_BOUND(el, f.nel, 14)) return;
  const int64_t e0 = fl_at(el, 0, 25);  // the element's value 0 of a 25-value array
  float chi[25];
#pragma unroll
  for (int q = 0; q < 25; ++q) {
    int64_t g = __ldg(f.gidx + e0 + q * kFlChunk);
    if (!AXG_BOUND(g, st.nglob, 14)) g = 0;
    float k = 0.f;
    chi[q] = fluid_predicted<MODE, KAHAN>(st, g, k);
  }
  const int32_t info = __ldg(f.elinfo + el);
  int axslot = (info & 0xFFFFFF) - 1;
  if (axslot >= 0 && !AXG_BOUND((int64_t)axslot * 5 + 4, f.n_m0, 14)) axslot = -1;
  const int srcslot = ((info >> 24) & 0xF) - 1;
  const bool ax = axslot >= 0;
  const float *met = f.metric + fl_at(el, 0, (NONMONO ? 4 : 3) * 25);
  float loc[25];
  if (ax) {
    if (NONMONO)
#pragma unroll
      for (int j = 0; j < 5; ++j) chi[5 * j] = 0.f;  // apply_axis_mask_scal(chi)
    fluid_elem_stiffness<true, NONMONO != 0>(sp, met, f.m0 + (int64_t)axslot * 5, chi, loc);
  } else {
    fluid_elem_stiffness<false, NONMONO != 0>(sp, met, nullptr, chi, loc);
  }
  if (srcslot >= 0 && f.srcfl) {
    const float stf1 = AXG_BOUND(*st.iter - 1, st.niter, 14) ? st.stf[*st.iter - 1] : 0.f;
    if (stf1 != 0.f)
#pragma unroll
      for (int q = 0; q < 25; ++q) loc[q] = loc[q] - f.srcfl[srcslot * 25 + q] * stf1;
  }
  if (NONMONO && ax)
#pragma unroll
    for (int j = 0; j < 5; ++j) loc[5 * j] = 0.f;
  if (f.fsmask)
#pragma unroll
    for (int q = 0; q < 25; ++q) loc[q] = loc[q] * __ldg(f.fsmask + e0 + q * kFlChunk);
#pragma unroll
  for (int q = 0; q < 25; ++q) f.fel[e0 + q * kFlChunk] = loc[q];
}

// Point pass: one thread per global point (items: the points of the
// solves).  The point's force is the coupling partial sum (if any) plus its
// copies' contributions in CSR order; then the corrector, as the last writer
// of the patch kernels applies it: ddchi = -inv_mass_fluid * force [-
// absorbing terms], dchi by the Newmark corrector or a symplectic kick, chi
// (zero on the axis for the non-monopole sources) and the next step's
// prediction stored.
template <int NONMONO, int MODE, bool KAHAN, class P = One<FluidWork>>
__global__ void __launch_bounds__(256) fluid_point_kernel(const __grid_constant__ P p) {
  pdl_wait();
  pdl_trigger();
  const int32_t it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= p.items()) return;
  const int sv = p.locate(it);
  const FluidArgs &f = p.at(sv).fa;
  const StateArgs &st = p.at(sv).st;
  if (*st.blowup) return;
  const int64_t g = it - p.first(sv);
  if (!AXG_BOUND(g, f.nglob, 15)) return;
  const uint32_t s0 = (uint32_t)f.start[g], s1 = (uint32_t)f.start[g + 1] & kFlStartMask;
  float sum = (s0 & kFlPartial) ? st.f[0][g] : 0.f;
  // the first four copies' indices, then their contributions, are loaded
  // together (an interior point has 1, 2 or 4 copies), then summed in order
  const int64_t nfel = fl_chunks(f.nel) * 25 * kFlChunk;
  uint32_t k = s0 & kFlStartMask;
  {
    int32_t e[4];
    float x[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      e[q] = k + q < s1 ? __ldg(f.ent + k + q) : -1;
      if (e[q] >= 0 && !AXG_BOUND(e[q], nfel, 15)) e[q] = -1;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) x[q] = e[q] >= 0 ? f.fel[e[q]] : 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (e[q] >= 0) sum = sum + x[q];
    k += 4;
  }
  for (; k < s1; ++k) {
    const int32_t e = __ldg(f.ent + k);
    if (!AXG_BOUND(e, nfel, 15)) break;
    sum = sum + f.fel[e];
  }
  float kc = 0.f;
  const float chi = fluid_predicted<MODE, KAHAN>(st, g, kc);
  const float vel = st.v[0][g];
  float a = -st.inv_mass[g] * sum;
  if (KAHAN && st.inv_mass_dp) a = (float)(-st.inv_mass_dp[g] * (double)sum);  // FP64, one rounding
  if (st.gamma) {
    const float gam = st.gamma[g];
    a = a - 2.f * gam * vel - gam * gam * chi;
  }
  float vn;
  if (MODE == MODE_SYMPLECTIC) {
    if (KAHAN) {
      float k = st.cv[0][g];
      vn = kahan_add(vel, mul2(st.kick, st.kick_lo, a), k);  // dchi + coefv(i) * ddchi, compensated
      st.cv[0][g] = k;
    } else {
      vn = vel + mul2(st.kick, st.kick_lo, a);  // dchi + coefv(i) * ddchi
    }
  } else if (KAHAN) {
    float k = st.cv[0][g];
    vn = kahan_add(vel, mul2(st.hdt, st.hdt_lo, st.a[0][g] + a), k);
    st.cv[0][g] = k;
  } else {
    vn = vel + mul2(st.hdt, st.hdt_lo, st.a[0][g] + a);
  }
  st.v[0][g] = vn;
  st.a[0][g] = a;
  // apply_axis_mask_scal zeroes chi on the axis (non-monopole)
  const bool zero = NONMONO && (s0 & kFlAxis);
  const float un = zero ? 0.f : chi;
  // plain Newmark: the new chi is the prediction read from up (axis points
  // stored as zero), which keeps it; st.u is the other buffer and receives
  // the next step's predictor
  if (MODE == MODE_NEWMARK && !KAHAN) st.u[0][g] = zero ? 0.f : predict(un, vn, a, st);
  else st.u[0][g] = un;
  if (KAHAN) st.cu[0][g] = zero ? 0.f : (MODE == MODE_NEWMARK ? comp_after_step(kc, vn, a, st) : kc);
}

// The final drift of a symplectic step (SOLVER/time_evol_wave.F90:722-727):
// chi += dchi * coefd(nstages+1), disp += velo * coefd(nstages+1), on every
// global point.
struct DriftWork {
  StateArgs solid, fluid;
  float cd, cd_lo;  // coefd(nstages + 1) deltat, an FP32 pair
};
template <class P = One<DriftWork>>
__global__ void drift_kernel(const __grid_constant__ P p) {
  const int32_t it = blockIdx.x * blockDim.x + threadIdx.x;  // a point of one of the solves
  if (it >= p.items()) return;
  const int sv = p.locate(it);
  const StateArgs &solid = p.at(sv).solid;
  const StateArgs &fluid = p.at(sv).fluid;
  const float cd = p.at(sv).cd, cd_lo = p.at(sv).cd_lo;
  if (*solid.blowup) return;
  const int64_t q = it - p.first(sv);
  // u + coefd(nstages+1) v; compensated where the handle keeps compensation
  auto drift = [&](float *u, const float *v, float *cu) {
    if (cu) {
      float k = cu[q];
      u[q] = kahan_add(u[q], mul2(cd, cd_lo, v[q]), k);
      cu[q] = k;
    } else {
      u[q] = u[q] + mul2(cd, cd_lo, v[q]);
    }
  };
  if (q < solid.nglob)
    for (int c = 0; c < 3; ++c)
      if (solid.u[c]) drift(solid.u[c], solid.v[c], solid.cu[c]);
  if (fluid.u[0] && q < fluid.nglob) drift(fluid.u[0], fluid.v[0], fluid.cu[0]);
}

// The plain Newmark step's predicted displacement up = disp + deltat*velo +
// half_dt_sq*acc0 (SOLVER/time_evol_wave.F90:357-364) of the current state,
// before a run: the last writers keep it from there on.  axmask (or null):
// per point, bit c set where the axis mask zeroes component c; those are
// stored as zero, as the step leaves them in its state.
__global__ void predict_kernel(StateArgs solid, const uint8_t *axmask) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= solid.nglob) return;
  const uint32_t m = axmask ? axmask[q] : 0u;
  for (int c = 0; c < 3; ++c)
    if (solid.up[c])
      solid.up[c][q] = ((m >> c) & 1u) ? 0.f : predict(solid.u[c][q], solid.v[c][q], solid.a[c][q], solid);
}

// ------------------------------------------------------------ coupling pre-passes

struct Coupling {
  // per boundary point (of the receiving domain): CSR of contributions
  const int32_t *pt_gidx;   // receiving global point
  const int32_t *start;     // n+1
  const int32_t *src_gidx;  // sending global point per contribution
  const float *b1, *b2;     // bdry_matr(ipol, b, 1/2) per contribution
  const float *mask;        // per contribution: 0 where the receiving copy is masked, else 1 (or fs mask)
  int32_t n;
  int64_t n_contrib, nglob_recv, nglob_send;  // extents (checked builds)
};

// bdry_copy2fluid (SOLVER/time_evol_wave.F90:1532-1571): fluid force starts
// with -(b1 * u_s [+ u_phi] + b2 * u_z) of the predicted solid displacement
struct ToFluidWork {
  Coupling cp;
  StateArgs solid;
  float *ffl;              // the fluid force partial sums
  const uint8_t *axmask;   // the solid's per-point axis mask bits (predict_kernel) or null
};
template <int DIPOLE, class P = One<ToFluidWork>>
__global__ void couple_to_fluid_kernel(const __grid_constant__ P p) {
  pdl_wait();
  pdl_trigger();
  const int32_t it = blockIdx.x * blockDim.x + threadIdx.x;  // a receiving point of one of the solves
  if (it >= p.items()) return;
  const int sv = p.locate(it);
  const Coupling &cp = p.at(sv).cp;
  const StateArgs &solid = p.at(sv).solid;
  float *ffl = p.at(sv).ffl;
  const uint8_t *axmask = p.at(sv).axmask;
  const int q = it - p.first(sv);
  if (*solid.blowup) return;
  if (q >= cp.n) return;
  float acc = 0.f;
  for (int k = cp.start[q]; k < cp.start[q + 1]; ++k) {
    if (!AXG_BOUND(k, cp.n_contrib, 21)) break;
    const int gs = cp.src_gidx[k];
    if (!AXG_BOUND(gs, cp.nglob_send, 21)) continue;
    // the same predicted displacement as the solid kernel's gather (plain
    // Newmark: the one the previous step's last writers stored)
    auto pred = [&](int c) {
      if (solid.cu[0]) {
        float k = solid.cu[c][gs];
        if (solid.stage) return drift_comp(solid.u[c][gs], solid.v[c][gs], solid, k);
        return predict_comp(solid.u[c][gs], solid.v[c][gs], solid.a[c][gs], solid, k);
      }
      if (solid.up[0]) {
        // the stored prediction has the axis-masked components zeroed; the
        // reference couples before its axis mask, with the prediction of the
        // masked (zero) displacement
        if (axmask && ((axmask[gs] >> c) & 1u)) return predict(0.f, solid.v[c][gs], solid.a[c][gs], solid);
        return solid.up[c][gs];
      }
      return predict(solid.u[c][gs], solid.v[c][gs], solid.a[c][gs], solid);
    };
    const float us = pred(0);
    const float uz = pred(2);
    float x = us;
    if (DIPOLE) x = us + pred(1);
    acc = acc + cp.mask[k] * (-cp.b1[k] * x - cp.b2[k] * uz);
  }
  if (AXG_BOUND(cp.pt_gidx[q], cp.nglob_recv, 22)) ffl[cp.pt_gidx[q]] = acc;
}

// bdry_copy2solid (SOLVER/time_evol_wave.F90:1577-1611): solid force starts
// with b1 * ddchi (s [and phi] components) and b2 * ddchi (z) of the new
// fluid acceleration; `mask` holds per contribution the axis mask bits.
struct ToSolidWork {
  Coupling cp;
  StateArgs fluid, solid;
};
template <int POLE, class P = One<ToSolidWork>>
__global__ void couple_to_solid_kernel(const __grid_constant__ P p) {
  pdl_wait();
  pdl_trigger();
  const int32_t it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= p.items()) return;
  const int sv = p.locate(it);
  const Coupling &cp = p.at(sv).cp;
  const StateArgs &fluid = p.at(sv).fluid;
  const StateArgs &solid = p.at(sv).solid;
  const int q = it - p.first(sv);
  if (*solid.blowup) return;
  if (q >= cp.n) return;
  float fs = 0.f, fp = 0.f, fz = 0.f;
  for (int k = cp.start[q]; k < cp.start[q + 1]; ++k) {
    if (!AXG_BOUND(k, cp.n_contrib, 23) || !AXG_BOUND(cp.src_gidx[k], cp.nglob_send, 23)) break;
    const float a = fluid.a[0][cp.src_gidx[k]];
    const bool masked = cp.mask[k] == 0.f;  // solid copy sits at ipol=0 of an axial element
    float ts = cp.b1[k] * a, tp = POLE == POLE_DI ? cp.b1[k] * a : 0.f, tz = cp.b2[k] * a;
    if (masked) {
      if (POLE == POLE_MONO) ts = 0.f;
      if (POLE == POLE_DI) { tp = 0.f; tz = 0.f; }
      if (POLE == POLE_QUAD) { ts = 0.f; tp = 0.f; tz = 0.f; }
    }
    fs = fs + ts;
    fp = fp + tp;
    fz = fz + tz;
  }
  const int g = cp.pt_gidx[q];
  if (!AXG_BOUND(g, cp.nglob_recv, 24)) return;
  solid.f[0][g] = fs;
  if (POLE != POLE_MONO) solid.f[1][g] = fp;
  solid.f[2][g] = fz;
}

// ------------------------------------------------------------ receivers, step counter

// nc_compute_recfile_seis_bare (SOLVER/seismograms.f90:783-820) every seis_it
// steps into rec(nseismo, 3, num_rec); advances the step counter afterwards.
// One CTA per solve.
struct RecWork {
  StateArgs solid;
  const int32_t *rec_gidx;
  int32_t num_rec, seis_it, pole, nseismo;
  float *rec;
  int32_t *iter_ctr;
};
template <class P = One<RecWork>>
__global__ void receivers_kernel(const __grid_constant__ P p) {
  pdl_wait();
  pdl_trigger();
  if ((int32_t)blockIdx.x >= p.items()) return;
  const RecWork &rw = p.at(p.locate(blockIdx.x));
  const StateArgs &solid = rw.solid;
  const int32_t *rec_gidx = rw.rec_gidx;
  const int32_t num_rec = rw.num_rec, seis_it = rw.seis_it, pole = rw.pole, nseismo = rw.nseismo;
  float *rec = rw.rec;
  int32_t *iter_ctr = rw.iter_ctr;
  const int32_t iter = *iter_ctr;
  __syncthreads();
  if (!*solid.blowup && seis_it > 0 && iter % seis_it == 0) {
    const int32_t is = iter / seis_it;
    if (is < nseismo) {
      for (int r = threadIdx.x; r < num_rec; r += blockDim.x) {
        const int g = rec_gidx[r];
        if (!AXG_BOUND(g, solid.nglob, 31)) continue;
        const float us = solid.u[0][g], uz = solid.u[2][g];
        const float up = pole == POLE_MONO ? 0.f : solid.u[1][g];
        float v1 = us, v2 = up, v3 = uz;
        if (pole == POLE_MONO) v2 = 0.f;
        if (pole == POLE_DI) { v1 = us + up; v2 = us - up; }
        const int64_t n = nseismo;
        rec[is + n * (0 + 3 * (int64_t)r)] = v1;
        rec[is + n * (1 + 3 * (int64_t)r)] = v2;
        rec[is + n * (2 + 3 * (int64_t)r)] = v3;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) *iter_ctr = iter + 1;
}

// ------------------------------------------------------------ kernel wavefield dumps

// dump_stuff (SOLVER/time_evol_wave.F90:1201-1249): the fields of one
// snapshot from the state at the end of a step.  One warp per element in the
// reference's element order, lane = GLL point (i, j); the gradients are the
// reference's axisym_gradient_* (SOLVER/pointwise_derivatives.f90:329-545)
// as shuffle contractions: mxm1 = G1T f (axial element) or G2T f, mxm2 = f G2,
// d/ds = dzdeta mxm1 + dzdxi mxm2, d/dz = dsdeta mxm1 + dsdxi mxm2.
enum { DUMP_DISPL_ONLY = 1, DUMP_STRAIN_ONLY = 2, DUMP_DISPL_VELO = 3, DUMP_FULLFIELDS = 4 };

struct DumpArgs {
  const int32_t *gidx;     // (25, nel): the element's points (0-based, internal numbering)
  const uint8_t *axial;    // per element: 1 on the axis
  const float *pw[5];      // DsDeta, DzDeta, DsDxi, DzDxi over J, 1/s: (25, nel)
  const float *inv_rho;    // fluid: 1/rho (25, nel)
  const float *u[3];       // solid disp (u[1] null for the monopole) / fluid chi (u[0])
  const float *v[3];       // solid velo / fluid dchi (v[0])
  float *out;              // the domain's first field
  int64_t nel, nglob;
  int32_t type, ibeg, iend, jbeg, jend;
  const int32_t *kwf;      // kernel wavefield layout: position of each element point (25, nel), -1: none; or null
  int64_t npt;             // points per field in that layout
  int32_t nsrcel;          // solid: elements whose values are dumped as zero (src_dump_type = 'mask')
  int32_t srcel[8];        // ... their 0-based indices
};

struct DumpLane {
  float dsdeta, dzdeta, dsdxi, dzdxi, inv_s;
};

// (d/ds f, d/dz f) at this lane; warp-uniform `ax`
__device__ __forceinline__ void dump_grad(const LaneCoef &c, const DumpLane &w, bool ax, int i, int j5, float f,
                                          float &gs, float &gz) {
  const float m1 = ax ? dxi(f, c.xi1, j5) : dxi(f, c.xi2, j5);
  const float m2 = deta(f, c.eta, i);
  gs = fmaf(w.dzdeta, m1, w.dzdxi * m2);
  gz = fmaf(w.dsdeta, m1, w.dsdxi * m2);
}

// f_over_s_*: f / s, and at the axis (i = 0 of an axial element) L'Hospital's
// df/ds (dsdf_*_allaxis, with G1T)
__device__ __forceinline__ float dump_fos(const LaneCoef &c, const DumpLane &w, bool ax, int i, int j5, float f) {
  float r = w.inv_s * f;
  if (ax) {
    const float m1 = dxi(f, c.xi1, j5), m2 = deta(f, c.eta, i);
    if (i == 0) r = fmaf(w.dzdeta, m1, w.dzdxi * m2);
  }
  return r;
}

template <int POLE, bool FLUID>
__global__ void __launch_bounds__(kThreads) wavefield_dump_kernel(DumpArgs a, SpecDev sp) {
  const int lane = threadIdx.x & 31;
  const bool active = lane < 25;
  const int ml = active ? lane : 24;  // idle lanes take part in the shuffles on point 24's data
  const int i = ml % 5, j = ml / 5, j5 = 5 * j;
  LaneCoef coef;
  load_coef(sp, i, j, coef);
  const int ni = a.iend - a.ibeg + 1, nj = a.jend - a.jbeg + 1;
  const int64_t np = (int64_t)ni * nj;
  const bool mine = active && i >= a.ibeg && i <= a.iend && j >= a.jbeg && j <= a.jend;
  const int64_t pidx = (i - a.ibeg) + (int64_t)ni * (j - a.jbeg);
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t e = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); e < a.nel; e += nwarps) {
    const int64_t q = 25 * e + ml;
    int32_t g = a.gidx[q];
    if (!AXG_BOUND(g, a.nglob, 41)) g = 0;
    const bool ax = a.axial[e] != 0;
    const DumpLane w{a.pw[0][q], a.pw[1][q], a.pw[2][q], a.pw[3][q], a.pw[4][q]};
    int fld = 0;
    const int32_t kpos = a.kwf && active ? a.kwf[q] : -1;
    // src_dump_type = 'mask': the source elements' solid values are zero
    // (eradicate_src_elem_values, SOLVER/wavefields_io.f90:1123-1153)
    bool masked = false;
    if (!FLUID)
      for (int k = 0; k < a.nsrcel && k < 8; ++k) masked = masked || a.srcel[k] == e;
    auto put = [&](float val) {
      if (masked) val = 0.f;
      if (a.kwf) {
        if (kpos >= 0 && AXG_BOUND(kpos, a.npt, 42)) a.out[fld * a.npt + kpos] = val;
      } else if (mine) {
        a.out[(fld * a.nel + e) * np + pidx] = val;
      }
      ++fld;
    };
    constexpr bool nonmono = POLE != POLE_MONO;
    if (!FLUID) {
      const float x1 = a.u[0][g], x2 = nonmono ? a.u[1][g] : 0.f, x3 = a.u[2][g];
      if (a.type == DUMP_STRAIN_ONLY || a.type == DUMP_FULLFIELDS) {
        // compute_strain, SOLVER/time_evol_wave.F90:1286-1345
        float g1, g2, h1, h2;
        dump_grad(coef, w, ax, i, j5, POLE == POLE_DI ? x1 + x2 : x1, g1, g2);  // dsus, dzus
        put(g1);
        dump_grad(coef, w, ax, i, j5, x3, h1, h2);                              // dsuz, dzuz
        const float n1 = (g2 + h1) / 2.f, n2 = g1 + h2;
        put(n1);                                                                // E31
        float buff;
        if (POLE == POLE_MONO) buff = dump_fos(coef, w, ax, i, j5, x1);
        else if (POLE == POLE_DI) buff = 2.f * dump_fos(coef, w, ax, i, j5, x2);
        else buff = dump_fos(coef, w, ax, i, j5, x1 - 2.f * x2);
        put(buff);                                                              // E22
        put(buff + n2);                                                         // Ekk
        if (POLE == POLE_DI) {
          float p1, p2;
          dump_grad(coef, w, ax, i, j5, x1 - x2, p1, p2);                       // dsup, dzup
          put(-dump_fos(coef, w, ax, i, j5, x2) - p1 / 2.f);                    // E12
          put(-(dump_fos(coef, w, ax, i, j5, x3) + p2) / 2.f);                  // E23
        } else if (POLE == POLE_QUAD) {
          float p1, p2;
          dump_grad(coef, w, ax, i, j5, x2, p1, p2);
          put(-dump_fos(coef, w, ax, i, j5, x1 + x2 / 2.f) - p1 / 2.f);
          put(-dump_fos(coef, w, ax, i, j5, x3) - p2 / 2.f);
        }
      }
      // dump_disp_global / dump_velo_global transform the dipole to (s, phi);
      // dump_disp / dump_velo_dchi write the state as it is
      const bool global = a.type != DUMP_DISPL_VELO;
      auto vec = [&](float y1, float y2, float y3) {
        put(global && POLE == POLE_DI ? y1 + y2 : y1);
        if (nonmono) put(global && POLE == POLE_DI ? y1 - y2 : y2);
        put(y3);
      };
      if (a.type == DUMP_DISPL_ONLY || a.type == DUMP_DISPL_VELO) vec(x1, x2, x3);
      if (a.type == DUMP_DISPL_VELO || a.type == DUMP_FULLFIELDS)
        vec(a.v[0][g], nonmono ? a.v[1][g] : 0.f, a.v[2][g]);
    } else {
      const float chi = a.u[0][g];
      const float irho = a.inv_rho[q];
      if (a.type == DUMP_DISPL_VELO) {
        put(chi);
        put(a.v[0][g]);
        continue;
      }
      if (a.type == DUMP_STRAIN_ONLY || a.type == DUMP_FULLFIELDS) {
        // SOLVER/time_evol_wave.F90:1347-1408: usz = grad(chi) / rho
        float c1, c2, g1, g2, h1, h2;
        dump_grad(coef, w, ax, i, j5, chi, c1, c2);
        const float us = c1 * irho, uz = c2 * irho;
        dump_grad(coef, w, ax, i, j5, us, g1, g2);
        put(g1);
        dump_grad(coef, w, ax, i, j5, uz, h1, h2);
        const float n1 = (g2 + h1) / 2.f, n2 = g1 + h2;
        put(n1);
        const float fs = dump_fos(coef, w, ax, i, j5, us);
        put(fs);
        put(fs + n2);
        if (POLE == POLE_DI) {
          put((-fs) / 2.f);
          put(dump_fos(coef, w, ax, i, j5, uz) / 2.f);
        } else if (POLE == POLE_QUAD) {
          put(-fs);
          put(-dump_fos(coef, w, ax, i, j5, uz));
        }
      }
      auto flu_vec = [&](float f) {  // inv_rho grad(f): s, phi (zero), z
        float c1, c2;
        dump_grad(coef, w, ax, i, j5, f, c1, c2);
        put(irho * c1);
        if (nonmono) put(0.f);
        put(irho * c2);
      };
      if (a.type == DUMP_DISPL_ONLY) flu_vec(chi);
      if (a.type == DUMP_FULLFIELDS) flu_vec(a.v[0][g]);
    }
  }
}

}  // namespace axg
