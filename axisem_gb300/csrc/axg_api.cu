// axg_api.cu -- the C-ABI of include/axisem_gb300.h.
//
// axg_create validates the descriptor, plans the patch colouring of the
// solid and fluid domains (axg_plan.cpp), packs the per-element data in
// launch order (one contiguous block of metric terms per element), builds the
// solid-fluid coupling tables and copies everything to HBM.  axg_run advances
// the Newmark loop of SOLVER/time_evol_wave.F90:353-500 with the kernels of
// axg_kernels.cuh, captured in CUDA graphs of `steps_per_graph` steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <utility>
#include <string>
#include <tuple>
#include <vector>

#include "axg_kernels.cuh"
#include "axg_plan.h"
#include "axisem_gb300.h"

using namespace axg;

namespace {

std::string g_create_error = "no error";

std::string fmt(const char *f, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, f);
  vsnprintf(buf, sizeof buf, f, ap);
  va_end(ap);
  return buf;
}

// metric array order of an element block (SOLID_TERMS_USED)
std::vector<int> solid_slots(int pole) {
  std::vector<int> s = {AXG_M_1,  AXG_M_2,  AXG_M_3,  AXG_M_4,  AXG_M_W1, AXG_M11S, AXG_M21S, AXG_M41S,
                        AXG_M12S, AXG_M22S, AXG_M32S, AXG_M42S, AXG_M11Z, AXG_M21Z, AXG_M41Z};
  if (pole == AXG_DIPOLE)
    s.insert(s.end(), {AXG_M_5, AXG_M_6, AXG_M_7, AXG_M_8, AXG_M_W2, AXG_M_W3, AXG_M13S, AXG_M33S, AXG_M43S});
  if (pole == AXG_QUADPOLE)
    s.insert(s.end(), {AXG_M_5, AXG_M_6, AXG_M_7, AXG_M_8, AXG_M_W2, AXG_M_W3, AXG_M_W4, AXG_M_W5,
                       AXG_M1PHI, AXG_M2PHI, AXG_M4PHI});
  return s;
}
std::vector<int> axial_slots(int pole) {
  if (pole == AXG_MONOPOLE) return {AXG_M0_W1, AXG_M0_W2, AXG_M0_W3};
  if (pole == AXG_DIPOLE)
    return {AXG_M0_W1, AXG_M0_W2, AXG_M0_W3, AXG_M0_W4, AXG_M0_W6, AXG_M0_W7, AXG_M0_W8, AXG_M0_W9, AXG_M0_W10};
  return {AXG_M0_W1, AXG_M0_W2, AXG_M0_W3, AXG_M0_W4, AXG_M0_W5, AXG_M0_W6};
}

struct DevBuf {
  void *p = nullptr;
  size_t n = 0;
};

struct DomainDev {
  PatchMeta *meta = nullptr;
  uint32_t *pts = nullptr;
  int32_t *elinfo = nullptr;
  // the fluid's two passes: element points (launch order), the CSR of each
  // point's copies (flags in start), the per-copy contributions (per solve)
  int32_t *gidx = nullptr, *start = nullptr, *ent = nullptr;
  float *fel = nullptr;
  float *metric = nullptr;
  float *m0 = nullptr;
  float *fsmask = nullptr;
  float *srcfl = nullptr;
  // per global point: bit c set where the pole's axis mask zeroes component
  // c (points on the axis), or null
  uint8_t *axmask = nullptr;
  int64_t n_m0 = 0;
};

// Device buffers of a mesh (element blocks, plans, masses, coupling tables,
// attenuation constants): owned jointly by every handle that solves on the
// mesh (axg_create_sharing), freed with the last of them.
struct MeshPool {
  std::vector<void *> allocs;
  int64_t bytes = 0;
  ~MeshPool() {
    for (void *p : allocs) cudaFree(p);
  }
};

struct CouplingHost {
  std::vector<int32_t> pt_gidx, start, src_gidx;
  std::vector<float> b1, b2, mask;
};

}  // namespace

struct axg_handle {
  // descriptor scalars
  int pole = 0, fluid_src = 0;
  int64_t nel_s = 0, nel_f = 0, nglob_s = 0, nglob_f = 0;
  int32_t niter = 0, seis_it = 1, num_rec = 0, nseismo = 0;
  bool absorbing = false;
  double dt = 0, magnitude = 0;
  // igloc in the plans' internal point numbering (DomainPlan::new_of_old):
  // every per-point table and device array of the handle uses it
  std::vector<int32_t> igloc_s, igloc_f, rec_gidx;
  std::vector<uint8_t> pre_s, pre_f;
  DomainPlan ps, pf;
  int patch_elems = 0, growth = -1;  // requested patch shape (0 / -1: tuned)
  int steps_per_graph = 16;
  // device
  int device = 0;
  cudaStream_t stream = nullptr;
  SpecDev spec{};
  std::vector<void *> allocs;
  int64_t dev_bytes = 0;
  DomainDev ds, df;
  float *su[3] = {}, *sv[3] = {}, *sa[3] = {}, *sf[3] = {};
  std::vector<int32_t> ielsrc;  // the source elements (0-based, solid or fluid as fluid_src says)
  // The plain Newmark step's predicted displacement (and chi): the last
  // writers store it into the buffer of the old displacement, and the step's
  // prediction becomes the new displacement, so the two buffers trade roles
  // (su <-> sup, fu <-> fup) after every such step; `parity` counts the
  // trades modulo 2 (step graphs are captured per parity).
  float *sup[3] = {};
  float *fup = nullptr;
  int parity = 0;
  float *fu = nullptr, *fv = nullptr, *fa = nullptr, *ff = nullptr;
  float *inv_mass_s = nullptr, *inv_mass_f = nullptr, *gamma_s = nullptr, *gamma_f = nullptr;
  // FP64 inverse masses (mesh) and source values (solve), when the descriptor had them
  double *inv_mass_s_dp = nullptr, *inv_mass_f_dp = nullptr, *src_val_dp_d = nullptr;
  float *stf = nullptr, *rec = nullptr;
  int32_t *iter = nullptr, *blowup = nullptr, *rec_gidx_d = nullptr;
  int32_t *src_gidx_d = nullptr;
  float *src_val_d = nullptr;
  int32_t n_src = 0;
  // gvec I/O in the reference's numbering (made on first use): the solid
  // plan's new_of_old, a 3-component staging buffer, a copy stream
  int32_t *gvec_perm = nullptr;
  float *gvec_stage = nullptr;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_io[5] = {};
  Coupling to_fluid{}, to_solid{};
  cudaGraphExec_t graph[2] = {};  // steps_per_graph steps, per parity
  int graph_steps[2] = {};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev_done = nullptr;  // end of the work axg_run_async queued
  bool pending = false;
  int num_sms = 1, solid_ctas = 1;
  int32_t *errw = nullptr;
  std::string err = "no error";
  int64_t kernels_per_step = 0, kernels_per_force = 0;
  int solid_ctas_step = 1;
  // time scheme: 0 Newmark (newmark2), else a symplectic scheme of nstages stages
  int scheme = 0, nstages = 0;
  std::vector<double> sym_cd, sym_cv;  // coefd(1:nstages+1) deltat, coefv(1:nstages) deltat
  float *stf_stages = nullptr;         // (niter, nstages): the stf at the stages' times
  // compensated (Kahan) time integration
  bool kahan = false;
  float *cu_s[3] = {}, *cv_s[3] = {}, *cu_f = nullptr, *cv_f = nullptr;
  // coarse-grained attenuation
  bool anel = false;       // coarse-grained (cg4) attenuation, fused into the solid kernel
  bool anel_full = false;  // attenuation at every GLL point (anel_full_kernel)
  float *fx = nullptr;     // ... its per-slot force terms for the next step
  int nsls = 0;
  AnelArgs an{};
  std::vector<int32_t> slot_of_elem_s;  // solid element -> launch slot
  int32_t *sym_gidx = nullptr;           // symplectic + attenuation: each launch slot's points
  uint8_t *sym_axial = nullptr;          // and axis flag
  // kernel wavefield dumps (axg_set_wavefield_dump)
  std::vector<uint8_t> axial_s, axial_f;  // per element (reference order): on the axis
  struct Dump {
    int type = 0, strain_it = 1, ibeg = 0, iend = 4, jbeg = 0, jend = 4, ns = 0, nf = 0;
    int64_t np = 25, floats = 0;  // points per element, floats per snapshot
    float *out = nullptr;
    int64_t capacity = 0;
    int32_t *gidx_s = nullptr, *gidx_f = nullptr;
    uint8_t *ax_s = nullptr, *ax_f = nullptr;
    float *pw_s[5] = {}, *pw_f[5] = {}, *inv_rho = nullptr;
    int32_t *kwf_s = nullptr, *kwf_f = nullptr;  // kernel wavefield layout: position of each element point or -1
    bool kwf = false;
    int64_t npt_s = 0, npt_f = 0;                // points per field in that layout
    bool src_mask = false;                       // src_dump_type = 'mask'
    float *slot[2] = {};
    int64_t slot_floats = 0;
    cudaEvent_t ev_dump[2] = {}, ev_copy[2] = {};
    std::vector<std::string> names;
  } dump;
  cudaGraphExec_t graph_dump[2] = {};  // strain_it steps, when that differs from steps_per_graph
  int graph_dump_steps[2] = {};
  // seismogram checkpoints: every check_it steps the final samples go to `out`
  struct Checkpoint {
    int32_t check_it = 0, cap = 0;
    float *out = nullptr;
    int32_t queued = 0;                                     // samples whose copies are queued
    std::deque<std::pair<cudaEvent_t, int32_t>> inflight;   // copy completions, oldest first
    int32_t done = 0;                                       // samples whose copies completed
    std::vector<cudaEvent_t> free_events;
  } ckpt;
  // mesh-level buffers, shared with the handles created from this one
  std::shared_ptr<MeshPool> mesh;
  bool in_mesh = false;  // allocations go to the mesh pool while set
};

namespace {

using Dump = axg_handle::Dump;
int checkpoint_progress(axg_handle *h);

int fail(axg_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  else g_create_error = msg;
  return code;
}

int cuda_fail(axg_handle *h, cudaError_t e, const char *what) {
  const int code = (e == cudaErrorMemoryAllocation) ? AXG_ERR_OOM : AXG_ERR_CUDA;
  return fail(h, code, fmt("%s: %s", what, cudaGetErrorString(e)));
}

#define CK(call)                                                   \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call);         \
  } while (0)

template <typename T>
int dalloc(axg_handle *h, T **p, size_t count) {
  *p = nullptr;
  if (count == 0) return AXG_OK;
  void *q = nullptr;
  // 256 bytes of tail padding: no kernel reads past an extent, the pad only
  // keeps a future vectorised tail load inside the allocation.  A solve's own
  // buffers are stream-ordered (cudaMallocAsync / cudaFreeAsync on its
  // stream): creating or destroying a solve then does not synchronise the
  // device, so other solves keep running.
  const bool mesh_level = h->in_mesh && h->mesh;
  cudaError_t e = mesh_level ? cudaMalloc(&q, count * sizeof(T) + 256)
                             : cudaMallocAsync(&q, count * sizeof(T) + 256, h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaMalloc");
  if (mesh_level) {
    h->mesh->allocs.push_back(q);
    h->mesh->bytes += (int64_t)(count * sizeof(T));
  } else {
    h->allocs.push_back(q);
  }
  h->dev_bytes += (int64_t)(count * sizeof(T));
  *p = (T *)q;
  return AXG_OK;
}

template <typename T>
int upload(axg_handle *h, T **p, const std::vector<T> &v) {
  int rc = dalloc(h, p, v.size());
  if (rc) return rc;
  if (v.empty()) return AXG_OK;
  if (h->in_mesh && h->mesh) CK(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  else CK(cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream));  // pageable: staged
  return AXG_OK;
}

// ---------------------------------------------------------------- validation

// The descriptor fields a stiffness + assembly reads: sizes, pole type, the
// solid numbering, the spectral matrices, the pole's solid metric arrays and
// the axial elements with their vectors.
int validate_stiffness(const axg_mesh_desc *d) {
  auto bad = [](const std::string &m) { return fail(nullptr, AXG_ERR_BAD_DESC, m); };
  if (!d) return bad("descriptor is NULL");
  if (d->abi_version != AXG_ABI_VERSION) return bad(fmt("abi_version %d, expected %d", d->abi_version, AXG_ABI_VERSION));
  if (d->npol != AXG_NPOL) return bad(fmt("npol = %d; only npol = 4 is supported", d->npol));
  if (d->src_type < 0 || d->src_type > 2) return bad("src_type must be monopole/dipole/quadpole (0..2)");
  if (d->nel_solid <= 0 || d->nglob_solid <= 0) return bad("nel_solid and nglob_solid must be positive");
  if (!d->igloc_solid) return bad("igloc_solid is NULL");
  if (!d->G0 || !d->G1 || !d->G2) return bad("spectral matrices G0, G1, G2 are required");
  for (int s : solid_slots(d->src_type))
    if (!d->m_solid[s]) return bad(fmt("solid metric array %d required by this pole type is NULL", s));
  if (d->naxel_solid < 0 || d->naxel_solid > d->nel_solid) return bad("naxel_solid out of range");
  if (d->naxel_solid > 0) {
    if (!d->ax_el_solid) return bad("ax_el_solid is NULL");
    for (int s : axial_slots(d->src_type))
      if (!d->m0_solid[s]) return bad(fmt("axial vector M0_w%d is NULL", s + 1));
    for (int k = 0; k < d->naxel_solid; ++k)
      if (d->ax_el_solid[k] < 1 || d->ax_el_solid[k] > d->nel_solid) return bad("ax_el_solid entry out of range");
  }
  return AXG_OK;
}

int validate(const axg_mesh_desc *d) {
  auto bad = [](const std::string &m) { return fail(nullptr, AXG_ERR_BAD_DESC, m); };
  if (!d) return bad("descriptor is NULL");
  if (d->abi_version != AXG_ABI_VERSION) return bad(fmt("abi_version %d, expected %d", d->abi_version, AXG_ABI_VERSION));
  if (d->npol != AXG_NPOL) return bad(fmt("npol = %d; only npol = 4 is supported", d->npol));
  if (d->src_type < 0 || d->src_type > 2) return bad("src_type must be monopole/dipole/quadpole (0..2)");
  if (d->nel_solid <= 0 || d->nglob_solid <= 0) return bad("nel_solid and nglob_solid must be positive");
  if (d->nel_fluid < 0 || d->nglob_fluid < 0) return bad("negative fluid sizes");
  if (d->nel_fluid > 0 && d->nglob_fluid <= 0) return bad("nglob_fluid must be positive with fluid elements");
  if (!d->igloc_solid) return bad("igloc_solid is NULL");
  if (d->nel_fluid > 0 && !d->igloc_fluid) return bad("igloc_fluid is NULL");
  if (!d->G0 || !d->G1 || !d->G1T || !d->G2 || !d->G2T) return bad("spectral matrices G0..G2T are required");
  for (int s : solid_slots(d->src_type))
    if (!d->m_solid[s]) return bad(fmt("solid metric array %d required by this pole type is NULL", s));
  if (d->naxel_solid < 0 || d->naxel_solid > d->nel_solid) return bad("naxel_solid out of range");
  if (d->naxel_solid > 0) {
    if (!d->ax_el_solid) return bad("ax_el_solid is NULL");
    for (int s : axial_slots(d->src_type))
      if (!d->m0_solid[s]) return bad(fmt("axial vector M0_w%d is NULL", s + 1));
    for (int k = 0; k < d->naxel_solid; ++k)
      if (d->ax_el_solid[k] < 1 || d->ax_el_solid[k] > d->nel_solid) return bad("ax_el_solid entry out of range");
  }
  if (!d->inv_mass_rho) return bad("inv_mass_rho is NULL");
  if (d->nel_fluid > 0) {
    for (int t = 0; t < (d->src_type == AXG_MONOPOLE ? 3 : 4); ++t)
      if (!d->m_fluid[t]) return bad(fmt("fluid metric array %d is NULL", t));
    if (!d->inv_mass_fluid) return bad("inv_mass_fluid is NULL");
    if (d->naxel_fluid < 0 || d->naxel_fluid > d->nel_fluid) return bad("naxel_fluid out of range");
    if (d->naxel_fluid > 0) {
      if (!d->ax_el_fluid) return bad("ax_el_fluid is NULL");
      for (int k = 0; k < d->naxel_fluid; ++k)
        if (d->ax_el_fluid[k] < 1 || d->ax_el_fluid[k] > d->nel_fluid) return bad("ax_el_fluid entry out of range");
      if (d->src_type != AXG_MONOPOLE && !d->m0_w_fl) return bad("M0_w_fl is NULL");
    }
  }
  if (d->nel_bdry < 0) return bad("nel_bdry < 0");
  if (d->nel_bdry > 0) {
    if (d->nel_fluid <= 0) return bad("solid-fluid boundary without fluid elements");
    if (!d->bdry_matr || !d->bdry_solid_el || !d->bdry_fluid_el || !d->bdry_jpol_solid || !d->bdry_jpol_fluid)
      return bad("boundary arrays are NULL");
    for (int b = 0; b < d->nel_bdry; ++b) {
      if (d->bdry_solid_el[b] < 1 || d->bdry_solid_el[b] > d->nel_solid) return bad("bdry_solid_el out of range");
      if (d->bdry_fluid_el[b] < 1 || d->bdry_fluid_el[b] > d->nel_fluid) return bad("bdry_fluid_el out of range");
      if (d->bdry_jpol_solid[b] < 0 || d->bdry_jpol_solid[b] > 4) return bad("bdry_jpol_solid out of range");
      if (d->bdry_jpol_fluid[b] < 0 || d->bdry_jpol_fluid[b] > 4) return bad("bdry_jpol_fluid out of range");
    }
  }
  if (d->nelsrc < 0 || d->nelsrc > 8) return bad("nelsrc must be within 0..8");
  if (d->nelsrc > 0) {
    if (!d->ielsrc) return bad("ielsrc is NULL");
    const int nmax = d->fluid_src ? d->nel_fluid : d->nel_solid;
    for (int k = 0; k < d->nelsrc; ++k)
      if (d->ielsrc[k] < 1 || d->ielsrc[k] > nmax) return bad("ielsrc entry out of range");
    if (d->fluid_src ? !d->source_term_fl : !d->source_term_el) return bad("source term array is NULL");
  }
  if (d->niter < 0) return bad("niter < 0");
  if (d->niter > 0 && !d->stf) return bad("stf is NULL");
  if (d->num_rec < 0) return bad("num_rec < 0");
  if (d->num_rec > 0) {
    if (!d->recfile_el) return bad("recfile_el is NULL");
    if (d->seis_it < 1) return bad("seis_it must be >= 1");
    for (int r = 0; r < d->num_rec; ++r) {
      const int e = d->recfile_el[r], ip = d->recfile_el[r + d->num_rec], jp = d->recfile_el[r + 2 * d->num_rec];
      if (e < 1 || e > d->nel_solid || ip < 0 || ip > 4 || jp < 0 || jp > 4) return bad("recfile_el entry out of range");
    }
  }
  if (d->have_absorbing_bc && (!d->solid_absorbing_gamma || (d->nel_fluid > 0 && !d->fluid_absorbing_gamma)))
    return bad("absorbing gamma arrays are NULL");
  if (!(d->deltat > 0) && d->niter > 0) return bad("deltat must be positive");
  if (d->anel_true) {
    if (d->att_coarse_grained != 0 && d->att_coarse_grained != 1) return bad("att_coarse_grained must be 0 or 1");
    if (d->n_sls < 1 || d->n_sls > kMaxSls)
      return fail(nullptr, AXG_ERR_UNSUPPORTED, fmt("n_sls = %d; 1..%d are supported", d->n_sls, kMaxSls));
    if (!d->y_j_attenuation || !d->exp_w_j_deltat || !d->ts_fac_t || !d->ts_fac_tm1 || !d->Q_mu || !d->Q_kappa ||
        !d->inv_s_solid)
      return bad("attenuation arrays are NULL");
    if (!d->att_coarse_grained &&
        (!d->delta_mu || !d->delta_kappa || !d->Y || !d->V_s_eta || !d->V_s_xi || !d->V_z_eta || !d->V_z_xi ||
         !d->Y0 || !d->V0_s_eta || !d->V0_s_xi || !d->V0_z_eta || !d->V0_z_xi || !d->DsDeta_over_J_sol ||
         !d->DzDeta_over_J_sol || !d->DsDxi_over_J_sol || !d->DzDxi_over_J_sol))
      return bad("attenuation arrays of every GLL point are NULL (att_coarse_grained = 0)");
    if (d->att_coarse_grained &&
        (!d->delta_mu_cg4 || !d->delta_kappa_cg4 || !d->Y_cg4 || !d->V_s_eta_cg4 || !d->V_s_xi_cg4 ||
         !d->V_z_eta_cg4 || !d->V_z_xi_cg4 || !d->DsDeta_over_J_sol_cg4 || !d->DzDeta_over_J_sol_cg4 ||
         !d->DsDxi_over_J_sol_cg4 || !d->DzDxi_over_J_sol_cg4))
      return bad("attenuation arrays are NULL");
    for (int64_t e = 0; e < d->nel_solid; ++e)
      if (!(d->Q_mu[e] > 0.f) || !(d->Q_kappa[e] > 0.f)) return bad("Q_mu and Q_kappa must be positive");
  }
  return AXG_OK;
}

// per global point value of an element-local array (first copy wins)
template <class T>
std::vector<T> per_point(const T *elem, const std::vector<int32_t> &igloc, int64_t nglob) {
  std::vector<T> out(nglob, T(0));
  std::vector<uint8_t> set(nglob, 0);
  for (size_t p = 0; p < igloc.size(); ++p) {
    const int64_t g = igloc[p] - 1;
    if (!set[g]) {
      out[g] = elem[p];
      set[g] = 1;
    }
  }
  return out;
}

// The fluid's arrays for its two passes.  mesh_part (mesh pool): the metric
// blocks, axial vectors and free-surface mask per element slot (launch
// order), the slots' global points, and per point the CSR of its copies with
// its flags (a coupling pre-pass partial sum; on the axis); always (this
// solve): the element info words (source slot), the fluid source terms and
// the per-copy contribution buffer.
int build_fluid_passes(axg_handle *h, const axg_mesh_desc *d, const std::vector<int32_t> &order, DomainDev &dd,
                       bool mesh_part, const std::vector<float> &metric, const std::vector<int32_t> &elinfo,
                       const std::vector<float> &m0, const std::vector<float> &fsmask, int nax, const int32_t *axl) {
  const int64_t nel = (int64_t)order.size(), nglob = h->nglob_f, nch = fl_chunks(nel);
  int rc;
  if (mesh_part) {
    if (nch * 25 * kFlChunk >= (int64_t)INT32_MAX) return fail(h, AXG_ERR_BAD_DESC, "fluid mesh too large");
    std::vector<int32_t> gidx((size_t)nch * 25 * kFlChunk, 0), start(nglob + 1, 0), ent((size_t)25 * nel);
    for (int64_t s = 0; s < nel; ++s) {
      const int64_t e = order[s];
      for (int k = 0; k < 25; ++k) {
        const int32_t g = h->igloc_f[25 * e + k] - 1;  // internal numbering
        gidx[fl_at(s, k, 25)] = g;
        start[g + 1]++;
      }
    }
    for (int64_t g = 0; g < nglob; ++g) start[g + 1] += start[g];
    if (start[nglob] >= (int64_t)kFlStartMask) return fail(h, AXG_ERR_BAD_DESC, "fluid mesh too large");
    {
      // copies in slot order: each point's contributions are summed in the
      // order of its elements' slots
      std::vector<int32_t> fill(start.begin(), start.end() - 1);
      for (int64_t s = 0; s < nel; ++s)
        for (int k = 0; k < 25; ++k) {
          const int64_t c = fl_at(s, k, 25);
          ent[fill[gidx[c]]++] = (int32_t)c;
        }
    }
    // flags: the coupling pre-pass's receiving points, the points on the axis
    for (size_t g = 0; g < h->pre_f.size(); ++g)
      if (h->pre_f[g]) start[h->pf.new_of_old[g]] |= (int32_t)kFlPartial;
    for (int k = 0; k < nax; ++k)
      for (int jj = 0; jj < 5; ++jj) start[h->igloc_f[25 * (int64_t)(axl[k] - 1) + 5 * jj] - 1] |= (int32_t)kFlAxis;
    // apply_axis_mask_scal (non-monopole sources) zeroes chi on the axis
    std::vector<uint8_t> axmask;
    if (d->src_type != AXG_MONOPOLE && nax > 0) {
      axmask.assign(nglob, 0);
      for (int64_t g = 0; g < nglob; ++g) axmask[g] = (start[g] & (int32_t)kFlAxis) ? 1 : 0;
    }
    h->in_mesh = true;
    rc = upload(h, &dd.metric, metric);
    if (!rc && !axmask.empty()) rc = upload(h, &dd.axmask, axmask);
    if (!rc) rc = upload(h, &dd.m0, m0);
    if (!rc && !fsmask.empty()) rc = upload(h, &dd.fsmask, fsmask);
    if (!rc) rc = upload(h, &dd.gidx, gidx);
    if (!rc) rc = upload(h, &dd.start, start);
    if (!rc) rc = upload(h, &dd.ent, ent);
    h->in_mesh = false;
    if (rc) return rc;
    dd.n_m0 = (int64_t)m0.size();
  }
  if ((rc = upload(h, &dd.elinfo, elinfo))) return rc;
  if ((rc = dalloc(h, &dd.fel, (size_t)nch * 25 * kFlChunk))) return rc;
  if (d->fluid_src && d->nelsrc > 0) {
    std::vector<float> s((size_t)8 * 25, 0.f);
    for (int k = 0; k < d->nelsrc; ++k)
      for (int q = 0; q < 25; ++q) s[25 * k + q] = d->source_term_fl[q + 25 * k];
    if ((rc = upload(h, &dd.srcfl, s))) return rc;
  }
  return AXG_OK;
}

// mesh_part: the element blocks, patch metadata and axial vectors (mesh
// pool); always: the point words (source and axis flags) and element info
// words of this solve.  The fluid's arrays: build_fluid_passes.
int build_domain(axg_handle *h, const axg_mesh_desc *d, bool fluid, bool mesh_part) {
  const DomainPlan &pl = fluid ? h->pf : h->ps;
  DomainDev &dd = fluid ? h->df : h->ds;
  const int64_t nel = pl.nel;
  if (nel == 0) return AXG_OK;
  const int pole = d->src_type;
  const int nonmono = pole != AXG_MONOPOLE;
  // axial flags and slots
  std::vector<uint8_t> axial(nel, 0);
  const int nax = fluid ? d->naxel_fluid : d->naxel_solid;
  const int32_t *axl = fluid ? d->ax_el_fluid : d->ax_el_solid;
  for (int k = 0; k < nax; ++k) axial[axl[k] - 1] = 1;
  std::vector<int> slots;
  int nt;
  if (fluid) {
    nt = nonmono ? 4 : 3;
  } else {
    slots = solid_slots(pole);
    nt = (int)slots.size();
  }
  // solid blocks carry the element's point indices and info word inline; the
  // fluid's element arrays are chunked (fl_at), its slots the plan's launch
  // order with the axial elements moved to the end, so that the element
  // pass's warps of 32 slots seldom mix axial and other elements
  const int bs = fluid ? 25 * nt : solid_block_stride(nt);
  const int64_t nslots = fluid ? fl_chunks(nel) * kFlChunk : nel;
  std::vector<float> metric(mesh_part ? (size_t)nslots * bs : 0, 0.f);
  std::vector<int32_t> elinfo(nel, 0);
  const std::vector<int> aslots = fluid ? std::vector<int>{0} : axial_slots(pole);
  const int na = (int)aslots.size();
  std::vector<float> m0;
  std::vector<float> fsmask;
  const bool use_fs = fluid && d->fluid_free_surface_mask != nullptr;
  if (use_fs && mesh_part) fsmask.resize((size_t)nslots * 25);
  // source slot of each element
  std::vector<int8_t> srcslot(nel, -1);
  if (d->nelsrc > 0 && (bool)d->fluid_src == fluid)
    for (int k = 0; k < d->nelsrc; ++k) srcslot[d->ielsrc[k] - 1] = (int8_t)k;
  std::vector<int32_t> order = pl.elem_order;
  if (fluid) std::stable_partition(order.begin(), order.end(), [&](int32_t e) { return !axial[e]; });
  int32_t axcount = 0;
  for (int64_t s = 0; s < nel; ++s) {
    const int64_t e = order[s];
    int32_t info = 0;
    if (axial[e]) {
      info = axcount + 1;
      if (mesh_part)
        for (int q = 0; q < na; ++q)
          for (int jj = 0; jj < 5; ++jj)
            m0.push_back(fluid ? (nonmono ? d->m0_w_fl[5 * e + jj] : 0.f) : d->m0_solid[aslots[q]][5 * e + jj]);
      ++axcount;
    }
    if (srcslot[e] >= 0) info |= (srcslot[e] + 1) << 24;
    elinfo[s] = info;
    if (!mesh_part) continue;
    if (fluid) {
      for (int t = 0; t < nt; ++t)
        for (int q = 0; q < 25; ++q) metric[fl_at(s, 25 * t + q, bs)] = d->m_fluid[t][25 * e + q];
      if (use_fs)
        for (int q = 0; q < 25; ++q) fsmask[fl_at(s, q, 25)] = d->fluid_free_surface_mask[25 * e + q];
      continue;
    }
    float *blk = metric.data() + (size_t)s * bs;
    for (int t = 0; t < nt; ++t) std::memcpy(blk + 25 * t, d->m_solid[slots[t]] + 25 * e, 25 * sizeof(float));
    {
      // the solid kernel reads only the axial slot of this info word
      std::memcpy(blk + solid_idx_off(nt), &pl.elem_pts[25 * s], 25 * sizeof(uint16_t));
      std::memcpy(blk + solid_info_off(nt), &info, sizeof(int32_t));
    }
  }
  if (fluid) return build_fluid_passes(h, d, order, dd, mesh_part, metric, elinfo, m0, fsmask, nax, axl);
  std::vector<uint32_t> pts = pl.pt_words;
  {
    // points on the axis: the last writer stores their masked components as
    // zero, as the reference's axis masks leave its state
    std::vector<uint8_t> onaxis(fluid ? h->nglob_f : h->nglob_s, 0);
    const std::vector<int32_t> &ig = fluid ? h->igloc_f : h->igloc_s;
    for (int k = 0; k < nax; ++k)
      for (int jj = 0; jj < 5; ++jj) onaxis[ig[25 * (int64_t)(axl[k] - 1) + 5 * jj] - 1] = 1;
    for (auto &w : pts)
      if (w != kPtPad && onaxis[w & kPtIndexMask]) w |= kPtAxis;
    if (mesh_part && nax > 0) {
      // the components the pole's axis mask zeroes (axis_masked)
      const uint8_t bits = pole == AXG_MONOPOLE ? 1 : pole == AXG_DIPOLE ? 6 : 7;
      for (auto &x : onaxis) x = x ? bits : 0;
      h->in_mesh = true;
      const int rc = upload(h, &dd.axmask, onaxis);
      h->in_mesh = false;
      if (rc) return rc;
    }
  }
  if (!fluid && h->n_src > 0) {
    // mark the points that carry a solid source term
    std::vector<uint8_t> issrc(h->nglob_s, 0);
    // the host copy of the source table is rebuilt here from the descriptor
    for (int k = 0; k < d->nelsrc; ++k) {
      const int64_t e = d->ielsrc[k] - 1;
      for (int q = 0; q < 25; ++q) {
        bool nz = false;
        for (int c = 0; c < 3; ++c) nz |= d->source_term_el[q + 25 * k + 200 * c] != 0.f;
        if (nz) issrc[h->igloc_s[25 * e + q] - 1] = 1;
      }
    }
    for (auto &w : pts)
      if (w != kPtPad && issrc[w & kPtIndexMask]) w |= kPtSource;
  }
  int rc;
  if (mesh_part) {
    h->in_mesh = true;
    if ((rc = upload(h, &dd.meta, pl.meta)) ||
        (rc = upload(h, &dd.metric, metric)) || (rc = upload(h, &dd.m0, m0)) ||
        (use_fs && (rc = upload(h, &dd.fsmask, fsmask)))) {
      h->in_mesh = false;
      return rc;
    }
    h->in_mesh = false;
    dd.n_m0 = (int64_t)m0.size();
  }
  if ((rc = upload(h, &dd.pts, pts))) return rc;
  if ((rc = upload(h, &dd.elinfo, elinfo))) return rc;
  return AXG_OK;
}

int upload_coupling(axg_handle *h, const CouplingHost &c, Coupling &out) {
  out.n = (int32_t)c.pt_gidx.size();
  int rc;
  int32_t *pg, *st, *sg;
  float *b1, *b2, *mk;
  if ((rc = upload(h, &pg, c.pt_gidx))) return rc;
  if ((rc = upload(h, &st, c.start))) return rc;
  if ((rc = upload(h, &sg, c.src_gidx))) return rc;
  if ((rc = upload(h, &b1, c.b1))) return rc;
  if ((rc = upload(h, &b2, c.b2))) return rc;
  if ((rc = upload(h, &mk, c.mask))) return rc;
  out.pt_gidx = pg;
  out.start = st;
  out.src_gidx = sg;
  out.b1 = b1;
  out.b2 = b2;
  out.mask = mk;
  out.n_contrib = (int64_t)c.src_gidx.size();
  return AXG_OK;
}

// group (receiver point, contribution) pairs by receiving point, keeping the
// boundary-list order inside each group
CouplingHost make_coupling(std::vector<std::tuple<int32_t, int32_t, float, float, float>> &v) {
  std::stable_sort(v.begin(), v.end(),
                   [](const auto &a, const auto &b) { return std::get<0>(a) < std::get<0>(b); });
  CouplingHost c;
  for (size_t k = 0; k < v.size(); ++k) {
    if (k == 0 || std::get<0>(v[k]) != std::get<0>(v[k - 1])) {
      c.pt_gidx.push_back(std::get<0>(v[k]));
      c.start.push_back((int32_t)k);
    }
    c.src_gidx.push_back(std::get<1>(v[k]));
    c.b1.push_back(std::get<2>(v[k]));
    c.b2.push_back(std::get<3>(v[k]));
    c.mask.push_back(std::get<4>(v[k]));
  }
  c.start.push_back((int32_t)v.size());
  return c;
}

// the plain Newmark step: its gather reads the predicted displacement the
// previous step's last writers stored
bool lookahead(const axg_handle *h) { return h->scheme == AXG_SCHEME_NEWMARK2 && !h->kahan; }

// after a plain Newmark step is queued: its prediction buffers hold the new
// displacement and chi, the old displacement buffers the next prediction
void trade_buffers(axg_handle *h) {
  if (!lookahead(h)) return;
  for (int c = 0; c < 3; ++c) std::swap(h->su[c], h->sup[c]);
  std::swap(h->fu, h->fup);
  h->parity ^= 1;
}

// Back to parity 0 (the allocation's roles): the state is copied into the
// first buffer (queued on s); the prediction is recomputed before a run.
cudaError_t normalize_buffers(axg_handle *h, cudaStream_t s) {
  if (!h->parity) return cudaSuccess;
  for (int c = 0; c < 3; ++c)
    if (h->su[c] && h->nglob_s > 0) {
      const cudaError_t e =
          cudaMemcpyAsync(h->sup[c], h->su[c], h->nglob_s * sizeof(float), cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return e;
      std::swap(h->su[c], h->sup[c]);
    }
  if (h->fu && h->nglob_f > 0) {
    const cudaError_t e = cudaMemcpyAsync(h->fup, h->fu, h->nglob_f * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    std::swap(h->fu, h->fup);
  }
  h->parity = 0;
  return cudaSuccess;
}

// an FP64 coefficient as an FP32 pair: hi = its FP32 rounding, lo = the rest
void split(double x, float &hi, float &lo) {
  hi = (float)x;
  lo = (float)(x - (double)hi);
}

StateArgs solid_state(axg_handle *h) {
  StateArgs s{};
  for (int c = 0; c < 3; ++c) {
    s.u[c] = h->su[c];
    s.v[c] = h->sv[c];
    s.a[c] = h->sa[c];
    s.f[c] = h->sf[c];
  }
  for (int c = 0; c < 3; ++c) {
    s.cu[c] = h->kahan ? h->cu_s[c] : nullptr;
    s.cv[c] = h->kahan ? h->cv_s[c] : nullptr;
    s.up[c] = lookahead(h) ? h->sup[c] : nullptr;
  }
  s.inv_mass = h->inv_mass_s;
  s.inv_mass_dp = h->kahan ? h->inv_mass_s_dp : nullptr;
  s.gamma = h->gamma_s;
  s.stf = h->stf;
  s.iter = h->iter;
  s.blowup = h->blowup;
  s.err = h->errw;
  s.thresh = (float)(10.0 * std::fabs(h->magnitude));
  split(h->dt, s.dt, s.dt_lo);
  split(0.5 * h->dt, s.hdt, s.hdt_lo);
  split(0.5 * h->dt * h->dt, s.hdt2, s.hdt2_lo);
  s.src.gidx = h->src_gidx_d;
  s.src.val = h->src_val_d;
  s.src.val_dp = h->kahan ? h->src_val_dp_d : nullptr;
  s.src.n = h->n_src;
  s.nglob = h->nglob_s;
  s.niter = std::max(h->niter, 1);
  return s;
}

StateArgs fluid_state(axg_handle *h) {
  StateArgs s = solid_state(h);
  for (int c = 0; c < 3; ++c) s.u[c] = s.v[c] = s.a[c] = s.f[c] = s.cu[c] = s.cv[c] = s.up[c] = nullptr;
  s.cu[0] = h->kahan ? h->cu_f : nullptr;
  s.cv[0] = h->kahan ? h->cv_f : nullptr;
  s.u[0] = h->fu;
  s.up[0] = lookahead(h) ? h->fup : nullptr;
  s.v[0] = h->fv;
  s.a[0] = h->fa;
  s.f[0] = h->ff;
  s.inv_mass = h->inv_mass_f;
  s.inv_mass_dp = h->kahan ? h->inv_mass_f_dp : nullptr;
  s.gamma = h->gamma_f;
  s.src.n = 0;
  s.nglob = h->nglob_f;
  return s;
}

// Before a run of the plain Newmark step: the predicted displacement of the
// current state (it may have been set, reset, restored or advanced by
// another scheme or mode since the last run).  The last writers keep it from
// there on; recomputing it is exact, so runs in pieces match one run.
void launch_anel_full(axg_handle *h, cudaStream_t s, bool update);

cudaError_t refresh_predicted(axg_handle *h, cudaStream_t s) {
  if (h->anel_full && h->scheme == AXG_SCHEME_NEWMARK2) launch_anel_full(h, s, false);
  if (!lookahead(h)) return cudaGetLastError();
  if (h->nglob_s > 0)
    predict_kernel<<<(unsigned)((h->nglob_s + 255) / 256), 256, 0, s>>>(solid_state(h), h->ds.axmask);
  if (h->nel_f > 0)
    predict_kernel<<<(unsigned)((h->nglob_f + 255) / 256), 256, 0, s>>>(fluid_state(h), h->df.axmask);
  return cudaGetLastError();
}

RecWork rec_work(axg_handle *h, const StateArgs &ss) {
  return RecWork{ss, h->rec_gidx_d, h->num_rec, h->seis_it, h->pole, h->nseismo, h->rec, h->iter};
}

DomainArgs domain_args(const DomainDev &dd, const DomainPlan &pl) {
  DomainArgs a{};
  a.n_patches = pl.n_patches;
  a.n_pts = pl.total_pts;
  a.n_elem = pl.nel;
  a.n_m0 = dd.n_m0;
  a.meta = dd.meta;
  a.pts = dd.pts;
  a.elinfo = dd.elinfo;
  a.metric = dd.metric;
  a.m0 = dd.m0;
  a.fsmask = dd.fsmask;
  a.srcfl = dd.srcfl;
  return a;
}

template <int POLE, int MODE, bool ANEL, bool KAHAN = false>
constexpr int solid_smem_bytes() {
  constexpr int NC = POLE == POLE_MONO ? 2 : 3;
  return SolidSmem<NC, solid_block_stride(n_terms(POLE)), solid_stages(ANEL), ANEL ? kAnelSlot : 0,
                   solid_buffers(MODE, ANEL, KAHAN), solid_row(MODE, ANEL, KAHAN), KAHAN>::bytes;
}

// sets the kernel's shared-memory attributes; *ctas = resident CTAs on the GPU
template <class F>
int prepare_kernel_fn(axg_handle *h, F fn, int bytes, int *ctas) {
  CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  CK(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  int per_sm = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, bytes));
  if (per_sm < 1) return fail(h, AXG_ERR_CUDA, "solid kernel does not fit on an SM");
  *ctas = per_sm * h->num_sms;
  return AXG_OK;
}

template <int POLE, int MODE, bool ANEL, bool KAHAN>
int prepare_solid_kernel(axg_handle *h, int *ctas) {
  return prepare_kernel_fn(h, solid_patch_kernel<POLE, MODE, ANEL, KAHAN>,
                           solid_smem_bytes<POLE, MODE, ANEL, KAHAN>(), ctas);
}

// the stiffness kernel and the Newmark kernel the handle's modes select
template <int POLE>
int prepare_solid_kernels(axg_handle *h) {
  int rc = prepare_solid_kernel<POLE, MODE_FORCE, false, false>(h, &h->solid_ctas);
  if (rc) return rc;
  int *c = &h->solid_ctas_step;
  if (h->scheme != AXG_SCHEME_NEWMARK2) {
    if (h->anel)
      return h->kahan ? prepare_solid_kernel<POLE, MODE_SYMPLECTIC, true, true>(h, c)
                      : prepare_solid_kernel<POLE, MODE_SYMPLECTIC, true, false>(h, c);
    return h->kahan ? prepare_solid_kernel<POLE, MODE_SYMPLECTIC, false, true>(h, c)
                    : prepare_solid_kernel<POLE, MODE_SYMPLECTIC, false, false>(h, c);
  }
  if (h->anel) {
    return h->kahan ? prepare_solid_kernel<POLE, MODE_NEWMARK, true, true>(h, c)
                    : prepare_solid_kernel<POLE, MODE_NEWMARK, true, false>(h, c);
  }
  return h->kahan ? prepare_solid_kernel<POLE, MODE_NEWMARK, false, true>(h, c)
                  : prepare_solid_kernel<POLE, MODE_NEWMARK, false, false>(h, c);
}

int prepare_kernels(axg_handle *h) {
  if (h->pole == AXG_MONOPOLE) return prepare_solid_kernels<POLE_MONO>(h);
  if (h->pole == AXG_DIPOLE) return prepare_solid_kernels<POLE_DI>(h);
  return prepare_solid_kernels<POLE_QUAD>(h);
}

// A launch with programmatic stream serialization: the kernel may start
// while the one ahead of it in the stream finishes (it waits in pdl_wait()
// before reading what that kernel writes).  Used for the kernels of the
// stiffness step and of the Newmark step, which all call pdl_wait().
template <class... KArgs, class... Args>
void launch_pdl(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t s,
                Args &&...args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

template <int POLE, int MODE, bool ANEL, bool KAHAN>
void launch_solid_colours(axg_handle *h, cudaStream_t s) {
  DomainArgs a = domain_args(h->ds, h->ps);
  StateArgs st = solid_state(h);
  const int ctas = MODE == MODE_FORCE ? h->solid_ctas : h->solid_ctas_step;
  for (int c = 0; c < h->ps.n_colours; ++c) {
    a.patch_begin = h->ps.colour_start[c];
    const int n = h->ps.colour_start[c + 1] - h->ps.colour_start[c];
    const int grid = std::min(n, ctas);
    a.fx = MODE == MODE_NEWMARK && h->anel_full ? h->fx : nullptr;
    launch_pdl(solid_patch_kernel<POLE, MODE, ANEL, KAHAN>, grid, kThreads, solid_smem_bytes<POLE, MODE, ANEL, KAHAN>(),
               s, a, st, h->spec, n, h->an);
  }
}

template <int POLE, int MODE>
void launch_solid_pole(axg_handle *h, cudaStream_t s) {
  if (MODE == MODE_FORCE) {
    launch_solid_colours<POLE, MODE_FORCE, false, false>(h, s);
  } else if (h->anel) {
    if (h->kahan) launch_solid_colours<POLE, MODE_NEWMARK, true, true>(h, s);
    else launch_solid_colours<POLE, MODE_NEWMARK, true, false>(h, s);
  } else {
    if (h->kahan) launch_solid_colours<POLE, MODE_NEWMARK, false, true>(h, s);
    else launch_solid_colours<POLE, MODE_NEWMARK, false, false>(h, s);
  }
}

template <int MODE>
void launch_solid(axg_handle *h, cudaStream_t s) {
  if (h->pole == AXG_MONOPOLE) launch_solid_pole<POLE_MONO, MODE>(h, s);
  else if (h->pole == AXG_DIPOLE) launch_solid_pole<POLE_DI, MODE>(h, s);
  else launch_solid_pole<POLE_QUAD, MODE>(h, s);
}

__global__ void zero_points_kernel(const int32_t *gidx, int32_t n, float *f0, float *f1, float *f2) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int g = gidx[q];
  f0[g] = 0.f;
  if (f1) f1[g] = 0.f;
  f2[g] = 0.f;
}

FluidArgs fluid_args(axg_handle *h) {
  const DomainDev &dd = h->df;
  FluidArgs a{};
  a.gidx = dd.gidx;
  a.metric = dd.metric;
  a.elinfo = dd.elinfo;
  a.m0 = dd.m0;
  a.fsmask = dd.fsmask;
  a.srcfl = dd.srcfl;
  a.start = dd.start;
  a.ent = dd.ent;
  a.fel = dd.fel;
  a.nel = h->nel_f;
  a.nglob = h->nglob_f;
  a.n_m0 = dd.n_m0;
  return a;
}

// CTAs of the fluid's element pass: one thread per element
unsigned fluid_elem_grid(int64_t nel) {
  return (unsigned)std::max<int64_t>(1, (nel + kFlElemThreads - 1) / kFlElemThreads);
}

// The fluid of a Newmark step or a symplectic stage: the element pass, then
// the point pass.
template <int NONMONO, int MODE, bool KAHAN>
void launch_fluid_t(axg_handle *h, cudaStream_t s, const StateArgs &fs) {
  FluidArgs fa = fluid_args(h);
  if (MODE == MODE_SYMPLECTIC) fa.fsmask = nullptr;  // symplectic_time_loop applies no free-surface mask
  launch_pdl(fluid_elem_kernel<NONMONO, MODE, KAHAN, One<FluidWork>>, fluid_elem_grid(h->nel_f), kFlElemThreads, 0, s,
             One<FluidWork>{{fa, fs}, (int32_t)h->nel_f}, h->spec);
  launch_pdl(fluid_point_kernel<NONMONO, MODE, KAHAN, One<FluidWork>>, (unsigned)((h->nglob_f + 255) / 256), 256, 0,
             s, One<FluidWork>{{fa, fs}, (int32_t)h->nglob_f});
}
template <int MODE>
void launch_fluid(axg_handle *h, cudaStream_t s, const StateArgs &fs) {
  if (h->pole == AXG_MONOPOLE) {
    if (h->kahan) launch_fluid_t<0, MODE, true>(h, s, fs);
    else launch_fluid_t<0, MODE, false>(h, s, fs);
  } else {
    if (h->kahan) launch_fluid_t<1, MODE, true>(h, s, fs);
    else launch_fluid_t<1, MODE, false>(h, s, fs);
  }
}

// Attenuation at every GLL point: with update, the step's memory variables
// and the next step's force terms; without, the force terms of the current
// memory variables (before a run)
template <int POLE>
void launch_anel_full_pole(axg_handle *h, cudaStream_t s, bool update) {
  const FullAnelArgs fa{h->an, h->fx, h->sym_gidx, h->sym_axial, h->nel_s};
  const unsigned g = (unsigned)std::min<int64_t>((h->nel_s + kWarps - 1) / kWarps, 16 * (int64_t)h->num_sms);
  if (update) launch_pdl(anel_full_kernel<POLE, true>, g, kThreads, 0, s, fa, solid_state(h), h->spec);
  else anel_full_kernel<POLE, false><<<g, kThreads, 0, s>>>(fa, solid_state(h), h->spec);
}
void launch_anel_full(axg_handle *h, cudaStream_t s, bool update) {
  if (h->pole == AXG_MONOPOLE) launch_anel_full_pole<POLE_MONO>(h, s, update);
  else if (h->pole == AXG_DIPOLE) launch_anel_full_pole<POLE_DI>(h, s, update);
  else launch_anel_full_pole<POLE_QUAD>(h, s, update);
}

void enqueue_force(axg_handle *h, cudaStream_t s) {
  if (h->to_solid.n > 0)
    zero_points_kernel<<<(h->to_solid.n + 255) / 256, 256, 0, s>>>(h->to_solid.pt_gidx, h->to_solid.n, h->sf[0],
                                                                   h->sf[1], h->sf[2]);
  launch_solid<MODE_FORCE>(h, s);
}

void enqueue_step_symplectic(axg_handle *h, cudaStream_t s);

void enqueue_step(axg_handle *h, cudaStream_t s) {
  if (h->scheme != AXG_SCHEME_NEWMARK2) {
    enqueue_step_symplectic(h, s);
    return;
  }
  StateArgs ss = solid_state(h), fs = fluid_state(h);
  if (h->nel_f > 0) {
    if (h->to_fluid.n > 0) {
      const unsigned nb = (h->to_fluid.n + 255) / 256;
      const One<ToFluidWork> w{{h->to_fluid, ss, h->ff, h->ds.axmask}, h->to_fluid.n};
      if (h->pole == AXG_DIPOLE) launch_pdl(couple_to_fluid_kernel<1, One<ToFluidWork>>, nb, 256, 0, s, w);
      else launch_pdl(couple_to_fluid_kernel<0, One<ToFluidWork>>, nb, 256, 0, s, w);
    }
    launch_fluid<MODE_NEWMARK>(h, s, fs);
    if (h->to_solid.n > 0) {
      const unsigned nb = (h->to_solid.n + 255) / 256;
      const One<ToSolidWork> w{{h->to_solid, fs, ss}, h->to_solid.n};
      if (h->pole == AXG_MONOPOLE) launch_pdl(couple_to_solid_kernel<POLE_MONO, One<ToSolidWork>>, nb, 256, 0, s, w);
      else if (h->pole == AXG_DIPOLE) launch_pdl(couple_to_solid_kernel<POLE_DI, One<ToSolidWork>>, nb, 256, 0, s, w);
      else launch_pdl(couple_to_solid_kernel<POLE_QUAD, One<ToSolidWork>>, nb, 256, 0, s, w);
    }
  }
  launch_solid<MODE_NEWMARK>(h, s);
  trade_buffers(h);  // the state after the step
  if (h->anel_full) launch_anel_full(h, s, true);  // the memory variables from the stored displacement
  launch_pdl(receivers_kernel<One<RecWork>>, 1, 256, 0, s, One<RecWork>{rec_work(h, solid_state(h)), 1});
}

// One step of symplectic_time_loop (SOLVER/time_evol_wave.F90:587-727):
// per stage the drift (on the gathers), fluid stiffness and the coupling
// into it, solid stiffness, the coupling into the solid, the kicks (by the
// last writers); then the final drift and the seismograms.
template <int POLE, bool ANEL, bool KAHAN>
void launch_solid_symplectic_modes(axg_handle *h, cudaStream_t s, const StateArgs &st) {
  DomainArgs a = domain_args(h->ds, h->ps);
  for (int c = 0; c < h->ps.n_colours; ++c) {
    a.patch_begin = h->ps.colour_start[c];
    const int n = h->ps.colour_start[c + 1] - h->ps.colour_start[c];
    solid_patch_kernel<POLE, MODE_SYMPLECTIC, ANEL, KAHAN>
        <<<std::min(n, h->solid_ctas_step), kThreads, solid_smem_bytes<POLE, MODE_SYMPLECTIC, ANEL, KAHAN>(), s>>>(
            a, st, h->spec, n, h->an);
  }
}

template <int POLE>
void launch_solid_symplectic(axg_handle *h, cudaStream_t s, const StateArgs &st) {
  if (h->anel) {
    if (h->kahan) launch_solid_symplectic_modes<POLE, true, true>(h, s, st);
    else launch_solid_symplectic_modes<POLE, true, false>(h, s, st);
  } else {
    if (h->kahan) launch_solid_symplectic_modes<POLE, false, true>(h, s, st);
    else launch_solid_symplectic_modes<POLE, false, false>(h, s, st);
  }
}

// the solid and fluid state of stage i of a symplectic step
void symplectic_stage_states(axg_handle *h, int i, StateArgs &ss, StateArgs &fs) {
  ss = solid_state(h);
  fs = fluid_state(h);
  split(h->sym_cd[i], ss.dt, ss.dt_lo);
  split(h->sym_cv[i], ss.kick, ss.kick_lo);
  ss.hdt2 = ss.hdt2_lo = 0.f;  // the coupling's predictor is then the drift u + coefd(i) v
  ss.stage = fs.stage = 1;
  fs.dt = ss.dt;
  fs.dt_lo = ss.dt_lo;
  fs.kick = ss.kick;
  fs.kick_lo = ss.kick_lo;
  fs.hdt2 = fs.hdt2_lo = 0.f;
  ss.stf = h->stf_stages + (int64_t)i * std::max(h->niter, 1);
}

// the final drift of a symplectic step: one thread per point of the larger domain
DriftWork drift_work(axg_handle *h) {
  DriftWork w{solid_state(h), fluid_state(h), 0.f, 0.f};
  split(h->sym_cd[h->nstages], w.cd, w.cd_lo);
  return w;
}
int32_t drift_points(const axg_handle *h) {
  return (int32_t)std::max(h->nglob_s, h->nel_f > 0 ? h->nglob_f : 0);
}

template <int POLE>
void launch_anel_memvar(axg_handle *h, cudaStream_t s) {
  const unsigned g = (unsigned)std::min<int64_t>((h->nel_s + kWarps - 1) / kWarps, 16 * (int64_t)h->num_sms);
  anel_memvar_kernel<POLE><<<g, kThreads, 0, s>>>(h->an, h->sym_gidx, h->sym_axial, solid_state(h), h->nel_s,
                                                  h->spec);
}
// the memory variables from the drifted displacement, once per symplectic step
void launch_anel_memvar_pole(axg_handle *h, cudaStream_t s) {
  if (h->pole == AXG_MONOPOLE) launch_anel_memvar<POLE_MONO>(h, s);
  else if (h->pole == AXG_DIPOLE) launch_anel_memvar<POLE_DI>(h, s);
  else launch_anel_memvar<POLE_QUAD>(h, s);
}

void enqueue_step_symplectic(axg_handle *h, cudaStream_t s) {
  for (int i = 0; i < h->nstages; ++i) {
    StateArgs ss, fs;
    symplectic_stage_states(h, i, ss, fs);
    if (h->nel_f > 0) {
      if (h->to_fluid.n > 0) {
        const int nb = (h->to_fluid.n + 255) / 256;
        const One<ToFluidWork> w{{h->to_fluid, ss, h->ff, h->ds.axmask}, h->to_fluid.n};
        if (h->pole == AXG_DIPOLE) couple_to_fluid_kernel<1><<<nb, 256, 0, s>>>(w);
        else couple_to_fluid_kernel<0><<<nb, 256, 0, s>>>(w);
      }
      launch_fluid<MODE_SYMPLECTIC>(h, s, fs);
      if (h->to_solid.n > 0) {
        const int nb = (h->to_solid.n + 255) / 256;
        const One<ToSolidWork> w{{h->to_solid, fs, ss}, h->to_solid.n};
        if (h->pole == AXG_MONOPOLE) couple_to_solid_kernel<POLE_MONO><<<nb, 256, 0, s>>>(w);
        else if (h->pole == AXG_DIPOLE) couple_to_solid_kernel<POLE_DI><<<nb, 256, 0, s>>>(w);
        else couple_to_solid_kernel<POLE_QUAD><<<nb, 256, 0, s>>>(w);
      }
    }
    if (h->pole == AXG_MONOPOLE) launch_solid_symplectic<POLE_MONO>(h, s, ss);
    else if (h->pole == AXG_DIPOLE) launch_solid_symplectic<POLE_DI>(h, s, ss);
    else launch_solid_symplectic<POLE_QUAD>(h, s, ss);
  }
  const int32_t n = drift_points(h);
  drift_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(One<DriftWork>{drift_work(h), n});
  if (h->anel) launch_anel_memvar_pole(h, s);
  receivers_kernel<<<1, 256, 0, s>>>(One<RecWork>{rec_work(h, solid_state(h)), 1});
}

// a CUDA graph of nsteps steps into *exec (replacing what it held).  The
// capture trades the buffers of each plain Newmark step as queueing does; a
// failed capture leaves the handle's buffer roles as they were.
int build_graph_into(axg_handle *h, int nsteps, cudaGraphExec_t *exec) {
  if (*exec) {
    cudaGraphExecDestroy(*exec);
    *exec = nullptr;
  }
  const int parity0 = h->parity;
  auto undo = [&]() {
    if (h->parity != parity0) trade_buffers(h);
  };
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < nsteps; ++k) enqueue_step(h, h->stream);
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (e != cudaSuccess) {
    undo();
    return cuda_fail(h, e, "cudaStreamEndCapture");
  }
  e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    undo();
    return cuda_fail(h, e, "cudaGraphInstantiate");
  }
  return AXG_OK;
}

// Queues k steps as one graph of slots[parity] (captured on first use, which
// trades the buffers as it goes; a replay trades them here).
int launch_graph(axg_handle *h, int k, cudaGraphExec_t *slots, int *slot_steps) {
  const int p = h->parity;
  if (!slots[p] || slot_steps[p] != k) {
    slot_steps[p] = 0;
    const int rc = build_graph_into(h, k, &slots[p]);
    if (rc) return rc;
    slot_steps[p] = k;
  } else {
    for (int q = 0; q < (k & 1); ++q) trade_buffers(h);
  }
  CK(cudaGraphLaunch(slots[p], h->stream));
  return AXG_OK;
}

// the step graphs no longer match the handle's kernels or step count
void drop_graphs(axg_handle *h) {
  for (int p = 0; p < 2; ++p) {
    if (h->graph[p]) cudaGraphExecDestroy(h->graph[p]);
    if (h->graph_dump[p]) cudaGraphExecDestroy(h->graph_dump[p]);
    h->graph[p] = h->graph_dump[p] = nullptr;
    h->graph_steps[p] = h->graph_dump_steps[p] = 0;
  }
}

void release(axg_handle *h) {
  if (!h) return;
  drop_graphs(h);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->ev_done) cudaEventDestroy(h->ev_done);
  for (cudaEvent_t e : h->ev_io)
    if (e) cudaEventDestroy(e);
  for (int k = 0; k < 2; ++k) {
    if (h->dump.ev_dump[k]) cudaEventDestroy(h->dump.ev_dump[k]);
    if (h->dump.ev_copy[k]) cudaEventDestroy(h->dump.ev_copy[k]);
  }
  if (h->copy_stream) {
    cudaStreamSynchronize(h->copy_stream);
    cudaStreamDestroy(h->copy_stream);
  }
  for (auto &q : h->ckpt.inflight) cudaEventDestroy(q.first);
  for (cudaEvent_t e : h->ckpt.free_events) cudaEventDestroy(e);
  h->ckpt.inflight.clear();
  h->ckpt.free_events.clear();
  for (void *p : h->allocs) cudaFreeAsync(p, h->stream);
  if (h->stream) cudaStreamDestroy(h->stream);
  h->allocs.clear();
}

int state_ptrs(axg_handle *h, int field, float **p, int *nc, int64_t *nglob, bool *fluid) {
  *fluid = false;
  *nglob = h->nglob_s;
  *nc = 3;
  switch (field) {
    case AXG_FIELD_DISP: for (int c = 0; c < 3; ++c) p[c] = h->su[c]; return AXG_OK;
    case AXG_FIELD_VELO: for (int c = 0; c < 3; ++c) p[c] = h->sv[c]; return AXG_OK;
    case AXG_FIELD_ACC0: for (int c = 0; c < 3; ++c) p[c] = h->sa[c]; return AXG_OK;
    case AXG_FIELD_DISP_COMP:
    case AXG_FIELD_VELO_COMP:
      if (!h->cu_s[0]) return fail(h, AXG_ERR_BAD_ARG, "the compensated mode was never enabled on this handle");
      for (int c = 0; c < 3; ++c) p[c] = field == AXG_FIELD_DISP_COMP ? h->cu_s[c] : h->cv_s[c];
      return AXG_OK;
    default: break;
  }
  *fluid = true;
  *nglob = h->nglob_f;
  *nc = 1;
  switch (field) {
    case AXG_FIELD_CHI: p[0] = h->fu; return AXG_OK;
    case AXG_FIELD_DCHI: p[0] = h->fv; return AXG_OK;
    case AXG_FIELD_DDCHI0: p[0] = h->fa; return AXG_OK;
    case AXG_FIELD_CHI_COMP:
    case AXG_FIELD_DCHI_COMP:
      if (!h->cu_s[0]) return fail(h, AXG_ERR_BAD_ARG, "the compensated mode was never enabled on this handle");
      p[0] = field == AXG_FIELD_CHI_COMP ? h->cu_f : h->cv_f;
      return AXG_OK;
    default: break;
  }
  return fail(h, AXG_ERR_BAD_ARG, fmt("field %d not available", field));
}


// points written first by a coupling pre-pass (receiving side of bdry_copy2*)
void prepass_flags(const axg_mesh_desc *d, std::vector<uint8_t> &pre_s, std::vector<uint8_t> &pre_f) {
  pre_s.assign(d->nglob_solid, 0);
  pre_f.assign(d->nel_fluid > 0 ? d->nglob_fluid : 0, 0);
  for (int b = 0; b < d->nel_bdry; ++b) {
    const int64_t es = d->bdry_solid_el[b] - 1, ef = d->bdry_fluid_el[b] - 1;
    for (int i = 0; i < 5; ++i) {
      pre_s[d->igloc_solid[25 * es + i + 5 * d->bdry_jpol_solid[b]] - 1] = 1;
      pre_f[d->igloc_fluid[25 * ef + i + 5 * d->bdry_jpol_fluid[b]] - 1] = 1;
    }
  }
}

// Coefficients of the symplectic schemes (symplectic_coefficients,
// SOLVER/time_evol_wave.F90:749-967): coefd(1:n+1) drifts and coefv(1:n)
// kicks, in units of deltat.  The reference writes most of these constants
// without a kind suffix, so they are single-precision values widened to
// double (sp below); and its SS_scheme (:972-992) computes the middle drift
// as 1 / 2 - sum(...) in Fortran integer division (1 / 2 = 0) -- both are
// restated as it computes them.  Returns nstages, 0 for an unknown scheme.
double sp(double x) { return (double)(float)x; }
void ss_scheme(const std::vector<double> &g, std::vector<double> &a, std::vector<double> &b) {
  const int n = (int)g.size(), ns = 2 * n + 1;
  a.assign(ns + 1, 0.0);
  b.assign(ns, 0.0);
  a[0] = g[0] / 2.0;
  for (int i = 1; i < n; ++i) a[i] = (g[i - 1] + g[i]) / 2.0;
  double sa = 0.0;
  for (int i = 0; i < n; ++i) sa += a[i];
  a[n] = 0.0 - sa;  // 1 / 2 - sum(a(1:n)) with integer 1 / 2
  for (int i = n + 1; i <= 2 * n + 1; ++i) a[i] = a[2 * n + 1 - i];
  double sg = 0.0;
  for (int i = 0; i < n; ++i) b[i] = g[i], sg += g[i];
  b[n] = 1.0 - 2.0 * sg;
  for (int i = n + 1; i < 2 * n + 1; ++i) b[i] = b[2 * n - i];
}
int symplectic_coefficients(int scheme, std::vector<double> &cd, std::vector<double> &cv) {
  cd.clear();
  cv.clear();
  if (scheme == AXG_SCHEME_SYMPLEC4) {  // PEFRL (Omelyan, Mryglod and Folk, 2002)
    const double zeta = sp(+0.1786178958448091), iota = sp(-0.2123418310626054),
                 kappa = sp(-0.06626458266981849);
    cd = {zeta, kappa, 1.0 - 2.0 * (zeta + kappa), kappa, zeta};
    cv = {0.5 - iota, iota, iota, 0.5 - iota};
  } else if (scheme == AXG_SCHEME_ML_SO4M5) {  // McLachlan (1995), order 4, m = 5
    const double rho = (14.0 - std::sqrt(19.0)) / 108.0, theta = (20.0 - 7.0 * std::sqrt(19.0)) / 108.0;
    const double nu = 2.0 / 5.0, lambda = -1.0 / 10.0;
    cd = {rho, theta, 0.5 - rho - theta, 0.5 - rho - theta, theta, rho};
    cv = {nu, lambda, 1.0 - 2.0 * (nu + lambda), lambda, nu};
  } else if (scheme == AXG_SCHEME_ML_SO6M7) {  // McLachlan (1995), order 6, m = 7
    const double d[4] = {sp(-1.01308797891717472981), sp(1.18742957373254270702), sp(-0.01833585209646059034),
                         sp(0.34399425728109261313)};
    const double v[4] = {sp(0.00016600692650009894), sp(-0.37962421426377360608), sp(0.68913741185181063674),
                         sp(0.38064159097092574080)};
    cd = {d[0], d[1], d[2], d[3], d[3], d[2], d[1], d[0]};
    cv = {v[0], v[1], v[2], v[3], v[2], v[1], v[0]};
  } else if (scheme == AXG_SCHEME_KL_O8M17) {  // Kahan and Li (1997), order 8
    const double g[8] = {0.13020248308889008088, 0.56116298177510838456, -0.38947496264484728641,
                         0.15884190655515560090, -0.39590389413323757734, 0.18453964097831570709,
                         0.25837438768632204729, 0.29501172360931029887};
    std::vector<double> gv;
    for (double x : g) gv.push_back(sp(x));
    ss_scheme(gv, cd, cv);
  } else if (scheme == AXG_SCHEME_SS_35O10) {  // Sofroniou and Spaletta (2004), order 10
    const double g[17] = {0.078795722521686419263907679337684, 0.31309610341510852776481247192647,
                          0.027918383235078066109520273275299, -0.22959284159390709415121339679655,
                          0.13096206107716486317465685927961, -0.26973340565451071434460973222411,
                          0.074973343155891435666137105641410, 0.11199342399981020488957508073640,
                          0.36613344954622675119314812353150, -0.39910563013603589787862981058340,
                          0.10308739852747107731580277001372, 0.41143087395589023782070411897608,
                          -0.0048663605831352617621956593099771, -0.39203335370863990644808193642610,
                          0.051942502962449647037182904015976, 0.050665090759924496335874344156866,
                          0.049674370639729879054568800279461};
    std::vector<double> gv;
    for (double x : g) gv.push_back(sp(x));
    ss_scheme(gv, cd, cv);
  }
  return (int)cv.size();
}

// resident CTAs of the solid patch kernels on the current device (two per
// SM), which the patch tuner spreads a colour's patches over; 0 without a
// device
int solid_plan_ctas() {
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();  // (no device: the error is not the caller's)
    return 0;
  }
  return 2 * nsm;
}

// tuned (or requested) patch shape, then the plan; ctas: as solid_plan_ctas
// (0: the tuner assumes full launches); anel: the attenuated solid kernel
std::string plan_domain(const int32_t *igloc, int64_t nel, int64_t nglob, int patch_elems, int growth,
                        const std::vector<uint8_t> &prepass, DomainPlan &plan, bool renumber = true,
                        int ctas = 0, bool anel = false) {
  int pe = patch_elems, gr = growth;
  std::string e = tune_plan(igloc, nel, nglob, patch_elems, growth, &pe, &gr, ctas,
                            anel ? kPatchOverheadAnelastic : kPatchOverheadElastic);
  if (!e.empty()) return e;
  return build_plan(igloc, nel, nglob, pe, gr, prepass, plan, renumber);
}

int check_igloc(const int32_t *ig, int64_t n, int64_t nglob, const char *what) {
  for (int64_t p = 0; p < n; ++p)
    if (ig[p] < 1 || ig[p] > nglob) return fail(nullptr, AXG_ERR_BAD_DESC, fmt("%s entry outside 1..nglob", what));
  return AXG_OK;
}

// fast_correct (SOLVER/attenuation.f90:1139-1155): first-order correction of
// the linearised SLS weights, yp_j = y_j * dy_j
void sls_fast_correct(const double *y, double *yp, int n) {
  double dy = 1.0 + 0.5 * y[0];
  yp[0] = y[0] * dy;
  for (int k = 1; k < n; ++k) {
    dy = dy + (dy - 0.5) * y[k - 1] + 0.5 * y[k];
    yp[k] = y[k] * dy;
  }
}

// Attenuation tables of the time loop (SOLVER/attenuation.f90:81-202):
//  * per distinct Q value a row ts_fac_t(j) a_j(Q), ts_fac_tm1(j) a_j(Q), with
//    a_j = yp_j / sum(yp_j), yp_j = y_j / Q (fast_correct'ed when
//    do_corr_lowq), computed in double as the reference does (:113-131) and
//    rounded to float once;
//  * per element (launch order) the cg4 constants and the two row indices;
//  * the per-element state, zeroed by axg_reset.
// the element slots' points and axis flags (launch order), for the kernels
// that visit elements outside the patch kernel
int upload_slot_points(axg_handle *h) {
  if (h->sym_gidx) return AXG_OK;
  std::vector<int32_t> g(25 * (size_t)h->nel_s);
  std::vector<uint8_t> ax(h->nel_s);
  for (int64_t e = 0; e < h->nel_s; ++e) {
    const int64_t sl = h->slot_of_elem_s[e];
    for (int k = 0; k < 25; ++k) g[25 * sl + k] = h->igloc_s[25 * e + k] - 1;
    ax[sl] = h->axial_s[e];
  }
  int rc;
  if ((rc = upload(h, &h->sym_gidx, g)) || (rc = upload(h, &h->sym_axial, ax))) return rc;
  return AXG_OK;
}

// Attenuation at every GLL point: the per-slot constants (kFullConst
// floats), the state (memory variables and the previous step's sources in
// the reference's layouts), the force terms, the slots' points.
template <class RowFn>
int build_anel_full(axg_handle *h, const axg_mesh_desc *d, bool mesh_part, RowFn row, std::vector<float> &qtab,
                    const std::map<float, int32_t> &qrow) {
  const int nsls = d->n_sls;
  const int64_t nel = h->nel_s;
  const DomainPlan &pl = h->ps;
  std::vector<float> consts((size_t)nel * kFullConst, 0.f);
  const float *pt[12] = {d->delta_mu, d->delta_kappa, d->Y, d->V_s_eta, d->V_s_xi, d->V_z_eta, d->V_z_xi,
                         d->DsDeta_over_J_sol, d->DzDeta_over_J_sol, d->DsDxi_over_J_sol, d->DzDxi_over_J_sol,
                         d->inv_s_solid};
  const float *ax5[5] = {d->Y0, d->V0_s_eta, d->V0_s_xi, d->V0_z_eta, d->V0_z_xi};
  for (int64_t s = 0; s < nel; ++s) {
    const int64_t e = pl.elem_order[s];
    float *c = consts.data() + (size_t)s * kFullConst;
    for (int f = 0; f < 12; ++f) std::memcpy(c + 25 * f, pt[f] + 25 * e, 25 * sizeof(float));
    if (h->axial_s[e])
      for (int f = 0; f < 5; ++f) std::memcpy(c + F_Y0 + 5 * f, ax5[f] + 5 * e, 5 * sizeof(float));
    const int32_t qm = row(d->Q_mu[e]), qk = row(d->Q_kappa[e]);
    std::memcpy(c + F_QMU, &qm, 4);
    std::memcpy(c + F_QKA, &qk, 4);
  }
  h->nsls = nsls;
  h->an.nsls = nsls;
  h->an.state_stride = full_state_stride(nsls);
  h->an.n_q = (int32_t)qrow.size();
  for (int j = 0; j < kMaxSls; ++j) h->an.ex[j] = j < nsls ? (float)d->exp_w_j_deltat[j] : 0.f;
  h->slot_of_elem_s.assign(nel, 0);
  for (int64_t s = 0; s < nel; ++s) h->slot_of_elem_s[pl.elem_order[s]] = (int32_t)s;
  int rc;
  float *cp = nullptr, *qp = nullptr;
  if (mesh_part) {
    h->in_mesh = true;
    rc = upload(h, &cp, consts);
    h->in_mesh = false;
    if (rc) return rc;
    h->an.consts = cp;
  }
  if ((rc = upload(h, &qp, qtab))) return rc;
  h->an.qtab = qp;
  if ((rc = dalloc(h, &h->an.state, (size_t)nel * h->an.state_stride))) return rc;
  if ((rc = dalloc(h, &h->fx, (size_t)nel * 75))) return rc;
  return upload_slot_points(h);
}

int build_anel(axg_handle *h, const axg_mesh_desc *d, bool mesh_part) {
  const int nsls = d->n_sls;
  const int64_t nel = h->nel_s;
  const DomainPlan &pl = h->ps;
  std::map<float, int32_t> qrow;
  std::vector<float> qtab;
  auto row = [&](float Q) {
    auto it = qrow.find(Q);
    if (it != qrow.end()) return it->second;
    double y[kMaxSls], yp[kMaxSls], sum = 0.0;
    for (int j = 0; j < nsls; ++j) y[j] = d->y_j_attenuation[j] / (double)Q;
    if (d->do_corr_lowq) sls_fast_correct(y, yp, nsls);
    else for (int j = 0; j < nsls; ++j) yp[j] = y[j];
    for (int j = 0; j < nsls; ++j) sum += yp[j];
    const int32_t r = (int32_t)qrow.size();
    qtab.resize((size_t)(r + 1) * 2 * kMaxSls, 0.f);
    for (int j = 0; j < nsls; ++j) {
      const double a = yp[j] / sum;
      qtab[(size_t)r * 2 * kMaxSls + j] = (float)(d->ts_fac_t[j] * a);
      qtab[(size_t)r * 2 * kMaxSls + kMaxSls + j] = (float)(d->ts_fac_tm1[j] * a);
    }
    qrow[Q] = r;
    return r;
  };
  if (h->anel_full) return build_anel_full(h, d, mesh_part, row, qtab, qrow);
  std::vector<float> consts((size_t)nel * kAnelConst, 0.f);
  const float *fields[11] = {d->delta_mu_cg4, d->delta_kappa_cg4, d->Y_cg4,  d->V_s_eta_cg4,
                             d->V_s_xi_cg4,   d->V_z_eta_cg4,    d->V_z_xi_cg4, d->DsDeta_over_J_sol_cg4,
                             d->DzDeta_over_J_sol_cg4, d->DsDxi_over_J_sol_cg4, d->DzDxi_over_J_sol_cg4};
  const int cg_pt[4] = {1 + 5 * 1, 1 + 5 * 3, 3 + 5 * 1, 3 + 5 * 3};
  for (int64_t s = 0; s < nel; ++s) {
    const int64_t e = pl.elem_order[s];
    float *c = consts.data() + (size_t)s * kAnelConst;
    for (int f = 0; f < 11; ++f)
      for (int k = 0; k < 4; ++k) c[4 * f + k] = fields[f][4 * e + k];
    for (int k = 0; k < 4; ++k) c[A_INVS + k] = d->inv_s_solid[25 * e + cg_pt[k]];
    const int32_t qm = row(d->Q_mu[e]), qk = row(d->Q_kappa[e]);
    std::memcpy(c + A_QMU, &qm, 4);
    std::memcpy(c + A_QKA, &qk, 4);
  }
  h->nsls = nsls;
  h->an.nsls = nsls;
  h->an.state_stride = anel_state_stride(nsls);
  h->an.n_q = (int32_t)qrow.size();
  for (int j = 0; j < kMaxSls; ++j) h->an.ex[j] = j < nsls ? (float)d->exp_w_j_deltat[j] : 0.f;
  h->slot_of_elem_s.assign(nel, 0);
  for (int64_t s = 0; s < nel; ++s) h->slot_of_elem_s[pl.elem_order[s]] = (int32_t)s;
  int rc;
  float *cp = nullptr, *qp = nullptr;
  if (mesh_part) {  // the per-element constants belong to the mesh
    h->in_mesh = true;
    rc = upload(h, &cp, consts);
    h->in_mesh = false;
    if (rc) return rc;
    h->an.consts = cp;
  }
  if ((rc = upload(h, &qp, qtab))) return rc;  // depends on dt: this solve's
  h->an.qtab = qp;
  if ((rc = dalloc(h, &h->an.state, (size_t)nel * h->an.state_stride))) return rc;
  return AXG_OK;
}

}  // namespace

extern "C" int axg_reset(axg_handle *h);
extern "C" int axg_device_count(void);

namespace {
// share: an existing handle on the same mesh (axg_create_sharing) whose
// plans and mesh-level device buffers are used instead of building new ones
int create_impl(axg_handle *h, const axg_mesh_desc *d, const axg_handle *share = nullptr) {
  int rc = AXG_OK;
  h->pole = d->src_type;
  h->fluid_src = d->fluid_src;
  h->nel_s = d->nel_solid;
  h->nel_f = d->nel_fluid;
  h->nglob_s = d->nglob_solid;
  h->nglob_f = d->nglob_fluid;
  h->niter = d->niter;
  h->seis_it = d->seis_it > 0 ? d->seis_it : 1;
  h->num_rec = d->num_rec;
  h->nseismo = d->niter / h->seis_it + 1;
  h->absorbing = d->have_absorbing_bc != 0;
  h->dt = d->deltat;
  h->magnitude = d->magnitude;
  for (int k = 0; k < d->nelsrc; ++k) h->ielsrc.push_back(d->ielsrc[k] - 1);
  h->anel = d->anel_true != 0 && d->att_coarse_grained != 0;
  h->anel_full = d->anel_true != 0 && d->att_coarse_grained == 0;
  CouplingHost cf, cs;
  if (share) {
    // the same mesh: sizes, pole, numbering, axial elements, boundary and
    // attenuation layout must match (the metric terms are taken as equal)
    if (share->pole != h->pole || share->nel_s != h->nel_s || share->nel_f != h->nel_f ||
        share->nglob_s != h->nglob_s || share->nglob_f != h->nglob_f || share->absorbing != h->absorbing ||
        share->anel != h->anel || share->anel_full != h->anel_full ||
        ((h->anel || h->anel_full) && share->nsls != d->n_sls))
      return fail(h, AXG_ERR_BAD_DESC, "axg_create_sharing: the descriptor is not of the handle's mesh");
    // (the handle holds igloc in its internal numbering)
    auto same = [](const std::vector<int32_t> &mine, const int32_t *ig, int64_t n, int64_t nglob,
                   const std::vector<int32_t> &nofo) {
      for (int64_t p = 0; p < n; ++p)
        if (ig[p] < 1 || ig[p] > nglob || mine[p] != nofo[ig[p] - 1] + 1) return false;
      return true;
    };
    if (!same(share->igloc_s, d->igloc_solid, 25 * h->nel_s, h->nglob_s, share->ps.new_of_old) ||
        (h->nel_f > 0 && !same(share->igloc_f, d->igloc_fluid, 25 * h->nel_f, h->nglob_f, share->pf.new_of_old)))
      return fail(h, AXG_ERR_BAD_DESC, "axg_create_sharing: the global numbering differs from the handle's mesh");
    h->igloc_s = share->igloc_s;
    h->igloc_f = share->igloc_f;
    h->axial_s = share->axial_s;
    h->axial_f = share->axial_f;
    h->pre_s = share->pre_s;
    h->pre_f = share->pre_f;
    h->ps = share->ps;
    h->pf = share->pf;
    h->patch_elems = share->patch_elems;
    h->growth = share->growth;
  } else {
    h->igloc_s.assign(d->igloc_solid, d->igloc_solid + 25 * h->nel_s);
    if (h->nel_f > 0) h->igloc_f.assign(d->igloc_fluid, d->igloc_fluid + 25 * h->nel_f);
    for (int64_t p = 0; p < 25 * h->nel_s; ++p)
      if (h->igloc_s[p] < 1 || h->igloc_s[p] > h->nglob_s)
        return fail(h, AXG_ERR_BAD_DESC, "igloc_solid entry outside 1..nglob_solid");
    for (int64_t p = 0; p < 25 * h->nel_f; ++p)
      if (h->igloc_f[p] < 1 || h->igloc_f[p] > h->nglob_f)
        return fail(h, AXG_ERR_BAD_DESC, "igloc_fluid entry outside 1..nglob_fluid");
    // solid-fluid coupling tables (the receiving points are written first by a pre-pass)
    std::vector<std::tuple<int32_t, int32_t, float, float, float>> tf, ts;
    std::vector<uint8_t> axs(h->nel_s, 0), axf(h->nel_f > 0 ? h->nel_f : 1, 0);
    for (int k = 0; k < d->naxel_solid; ++k) axs[d->ax_el_solid[k] - 1] = 1;
    for (int k = 0; k < d->naxel_fluid; ++k) axf[d->ax_el_fluid[k] - 1] = 1;
    h->axial_s = axs;
    h->axial_f = axf;
    const int nb = d->nel_bdry;
    for (int b = 0; b < nb; ++b) {
      const int64_t es = d->bdry_solid_el[b] - 1, ef = d->bdry_fluid_el[b] - 1;
      const int js = d->bdry_jpol_solid[b], jf = d->bdry_jpol_fluid[b];
      for (int i = 0; i < 5; ++i) {
        const int32_t gs = h->igloc_s[25 * es + i + 5 * js] - 1;
        const int32_t gf = h->igloc_f[25 * ef + i + 5 * jf] - 1;
        const float b1 = d->bdry_matr[i + 5 * b], b2 = d->bdry_matr[i + 5 * (b + nb)];
        float mf = (d->src_type != AXG_MONOPOLE && axf[ef] && i == 0) ? 0.f : 1.f;
        if (d->fluid_free_surface_mask) mf *= d->fluid_free_surface_mask[25 * ef + i + 5 * jf];
        tf.emplace_back(gf, gs, b1, b2, mf);
        ts.emplace_back(gs, gf, b1, b2, (axs[es] && i == 0) ? 0.f : 1.f);
      }
    }
    cf = make_coupling(tf);
    cs = make_coupling(ts);
    h->pre_s.assign(h->nglob_s, 0);
    for (int32_t g : cs.pt_gidx) h->pre_s[g] = 1;
    if (h->nel_f > 0) {
      h->pre_f.assign(h->nglob_f, 0);
      for (int32_t g : cf.pt_gidx) h->pre_f[g] = 1;
    }
    std::string perr = plan_domain(h->igloc_s.data(), h->nel_s, h->nglob_s, h->patch_elems, h->growth, h->pre_s, h->ps,
                                   true, solid_plan_ctas(), h->anel);
    if (!perr.empty()) return fail(h, AXG_ERR_BAD_DESC, "solid plan: " + perr);
    if (h->nel_f > 0) {
      perr = plan_domain(h->igloc_f.data(), h->nel_f, h->nglob_f, h->patch_elems, h->growth, h->pre_f, h->pf);
      if (!perr.empty()) return fail(h, AXG_ERR_BAD_DESC, "fluid plan: " + perr);
    }
#ifdef AXG_VALIDATE_PLAN
    perr = validate_plan(h->igloc_s.data(), h->nel_s, h->nglob_s, h->pre_s, h->ps);
    if (!perr.empty()) return fail(h, AXG_ERR_BAD_DESC, "solid plan invalid: " + perr);
#endif
    // from here on points carry the plans' internal numbers
    for (int32_t &g : h->igloc_s) g = h->ps.new_of_old[g - 1] + 1;
    for (int32_t &g : h->igloc_f) g = h->pf.new_of_old[g - 1] + 1;
    for (int32_t &g : cs.pt_gidx) g = h->ps.new_of_old[g];
    for (int32_t &g : cs.src_gidx) g = h->pf.new_of_old[g];
    for (int32_t &g : cf.pt_gidx) g = h->pf.new_of_old[g];
    for (int32_t &g : cf.src_gidx) g = h->ps.new_of_old[g];
  }

  // receivers and the solid source table
  for (int r = 0; r < h->num_rec; ++r) {
    const int64_t e = d->recfile_el[r] - 1;
    const int ip = d->recfile_el[r + h->num_rec], jp = d->recfile_el[r + 2 * h->num_rec];
    h->rec_gidx.push_back(h->igloc_s[25 * e + ip + 5 * jp] - 1);
  }
  std::vector<int32_t> src_g;
  std::vector<float> src_v;
  std::vector<double> src_v_dp;
  if (!d->fluid_src) {
    std::map<int32_t, int> seen;
    for (int k = 0; k < d->nelsrc; ++k) {
      const int64_t e = d->ielsrc[k] - 1;
      for (int q = 0; q < 25; ++q) {
        float v[3];
        bool nz = false;
        for (int c = 0; c < 3; ++c) {
          v[c] = d->source_term_el[q + 25 * k + 200 * c];
          nz |= v[c] != 0.f;
        }
        const int32_t g = h->igloc_s[25 * e + q] - 1;
        if (!nz || seen.count(g)) continue;
        seen[g] = 1;
        src_g.push_back(g);
        src_v.insert(src_v.end(), v, v + 3);
        if (d->source_term_el_dp)
          for (int c = 0; c < 3; ++c) src_v_dp.push_back(d->source_term_el_dp[q + 25 * k + 200 * c]);
      }
    }
  }
  h->n_src = (int32_t)src_g.size();

  // ---- device
  CK(cudaGetDevice(&h->device));
  if (share && share->device != h->device)
    return fail(h, AXG_ERR_BAD_ARG, "axg_create_sharing: the handle's mesh is on another device");
  CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&h->ev0));
  CK(cudaEventCreate(&h->ev1));
  CK(cudaEventCreateWithFlags(&h->ev_done, cudaEventDisableTiming));
  for (int k = 0; k < 25; ++k) {
    h->spec.g1[k] = d->G1[k];
    h->spec.g2[k] = d->G2[k];
  }
  for (int k = 0; k < 5; ++k) h->spec.g0[k] = d->G0[k];
  CK(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device));
  if (share) {
    h->mesh = share->mesh;
    h->ds = share->ds;
    h->df = share->df;
    h->inv_mass_s = share->inv_mass_s;
    h->inv_mass_f = share->inv_mass_f;
    h->inv_mass_s_dp = share->inv_mass_s_dp;
    h->inv_mass_f_dp = share->inv_mass_f_dp;
    h->gamma_s = share->gamma_s;
    h->gamma_f = share->gamma_f;
    h->to_fluid = share->to_fluid;
    h->to_solid = share->to_solid;
    h->an.consts = share->an.consts;
    h->dev_bytes = h->mesh->bytes;
  } else {
    h->mesh = std::make_shared<MeshPool>();
    h->in_mesh = true;
    rc = upload(h, &h->inv_mass_s, per_point(d->inv_mass_rho, h->igloc_s, h->nglob_s));
    if (!rc && h->absorbing) rc = upload(h, &h->gamma_s, per_point(d->solid_absorbing_gamma, h->igloc_s, h->nglob_s));
    if (!rc && h->nel_f > 0) rc = upload(h, &h->inv_mass_f, per_point(d->inv_mass_fluid, h->igloc_f, h->nglob_f));
    if (!rc && d->inv_mass_rho_dp)
      rc = upload(h, &h->inv_mass_s_dp, per_point(d->inv_mass_rho_dp, h->igloc_s, h->nglob_s));
    if (!rc && h->nel_f > 0 && d->inv_mass_fluid_dp)
      rc = upload(h, &h->inv_mass_f_dp, per_point(d->inv_mass_fluid_dp, h->igloc_f, h->nglob_f));
    if (!rc && h->nel_f > 0 && h->absorbing)
      rc = upload(h, &h->gamma_f, per_point(d->fluid_absorbing_gamma, h->igloc_f, h->nglob_f));
    if (!rc) rc = upload_coupling(h, cf, h->to_fluid);
    if (!rc) rc = upload_coupling(h, cs, h->to_solid);
    h->in_mesh = false;
    if (rc) return rc;
    h->to_fluid.nglob_recv = h->nglob_f;
    h->to_fluid.nglob_send = h->nglob_s;
    h->to_solid.nglob_recv = h->nglob_s;
    h->to_solid.nglob_send = h->nglob_f;
  }
  if ((rc = build_domain(h, d, false, !share))) return rc;
  if ((rc = build_domain(h, d, true, !share))) return rc;
  const bool mono = h->pole == AXG_MONOPOLE;
  for (int c = 0; c < 3; ++c) {
    if (mono && c == 1) continue;
    if ((rc = dalloc(h, &h->su[c], h->nglob_s)) || (rc = dalloc(h, &h->sv[c], h->nglob_s)) ||
        (rc = dalloc(h, &h->sa[c], h->nglob_s)) || (rc = dalloc(h, &h->sf[c], h->nglob_s)) ||
        (rc = dalloc(h, &h->sup[c], h->nglob_s)))
      return rc;
  }
  if (h->nel_f > 0) {
    if ((rc = dalloc(h, &h->fu, h->nglob_f)) || (rc = dalloc(h, &h->fup, h->nglob_f)) ||
        (rc = dalloc(h, &h->fv, h->nglob_f)) ||
        (rc = dalloc(h, &h->fa, h->nglob_f)) || (rc = dalloc(h, &h->ff, h->nglob_f)))
      return rc;
  }
  std::vector<float> stf(d->stf ? d->stf : (const float *)nullptr, d->stf ? d->stf + d->niter : nullptr);
  if (stf.empty()) stf.assign(1, 0.f);
  if ((rc = upload(h, &h->stf, stf))) return rc;
  if ((rc = dalloc(h, &h->rec, (size_t)h->nseismo * 3 * std::max(h->num_rec, 1)))) return rc;
  if ((rc = upload(h, &h->rec_gidx_d, h->rec_gidx))) return rc;
  if ((rc = upload(h, &h->src_gidx_d, src_g))) return rc;
  if ((rc = upload(h, &h->src_val_d, src_v))) return rc;
  if (!src_v_dp.empty() && (rc = upload(h, &h->src_val_dp_d, src_v_dp))) return rc;
  if ((rc = dalloc(h, &h->iter, 4))) return rc;
  h->blowup = h->iter + 1;
  h->errw = h->iter + 2;
  if ((h->anel || h->anel_full) && (rc = build_anel(h, d, !share))) return rc;
  if ((rc = prepare_kernels(h))) return rc;
  h->kernels_per_force = h->ps.n_colours + (h->to_solid.n > 0 ? 1 : 0);
  h->kernels_per_step = h->ps.n_colours + 1 + (h->anel_full ? 1 : 0) +
                        (h->nel_f > 0 ? 2 + (h->to_fluid.n > 0) + (h->to_solid.n > 0) : 0);
  return axg_reset(h);
}
}  // namespace

// ============================================================== no-allocation variant
//
// Stiffness + assembly for callers that cannot allocate device memory: code
// running where cudaMalloc is unavailable or forbidden (inside another
// runtime's memory pool, a driver callback, a process whose device memory is
// fully reserved up front).  It runs the same planner and the same
// solid_patch_kernel<pole, FORCE> as axg_stiffness_assembled, but every
// device-side buffer -- plan, packed element blocks, u, f and control words --
// lives in one file-scope static device array of kNoAllocScratchBytes.  Each
// GPU that loads this library holds that array until the process exits.
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct NoAllocDevice {
  bool ready = false;
  unsigned long long ctx_id = 0;  // the CUDA context the set-up was made in
  unsigned char *base = nullptr;  // device address of g_noalloc_scratch on this device
  int grid_cap[3] = {0, 0, 0};    // resident CTAs of the FORCE kernel per pole
};
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];

template <int POLE>
int noalloc_prepare_kernel(int nsm, int *cap) {
  auto fn = solid_patch_kernel<POLE, MODE_FORCE, false, false>;
  const int bytes = solid_smem_bytes<POLE, MODE_FORCE, false, false>();
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  int per_sm = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, bytes);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "no-allocation set-up");
  *cap = std::max(per_sm, 1) * nsm;
  return AXG_OK;
}

// Id of the current CUDA context (cuCtxGetId, looked up through the runtime so
// that the library does not link the driver library); 0 when unavailable.
unsigned long long current_context_id() {
  typedef int (*CtxGetId)(void *, unsigned long long *);
  static CtxGetId fn = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetId>(p);
    looked_up = true;
  }
  unsigned long long id = 0;
  if (fn && fn(nullptr, &id) != 0) id = 0;
  return id;
}

// Once per device (and again when the device's context was replaced, e.g.
// after a cudaDeviceReset), with that device current: the symbol's device
// address and the kernel attributes.  The first call on a device makes this
// set-up; it should come before any stream capture.
int noalloc_setup(NoAllocDevice **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetDevice");
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(nullptr, AXG_ERR_UNSUPPORTED, "device ordinal too large");
  NoAllocDevice &nd = g_noalloc_dev[dev];
  const unsigned long long ctx = current_context_id();
  if (!nd.ready || ctx == 0 || ctx != nd.ctx_id) {
    nd.ready = false;
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    int nsm = 0;
    e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaDeviceGetAttribute");
    int rc;
    if ((rc = noalloc_prepare_kernel<POLE_MONO>(nsm, &nd.grid_cap[0])) ||
        (rc = noalloc_prepare_kernel<POLE_DI>(nsm, &nd.grid_cap[1])) ||
        (rc = noalloc_prepare_kernel<POLE_QUAD>(nsm, &nd.grid_cap[2])))
      return rc;
    nd.base = static_cast<unsigned char *>(ptr);
    nd.ctx_id = current_context_id();  // the symbol look-up made the context current if it was not
    nd.ready = nd.ctx_id != 0;         // without a context id the set-up is repeated on every call
  }
  *out = &nd;
  return AXG_OK;
}

template <int POLE>
void noalloc_launch(const DomainArgs &a0, const StateArgs &st, const SpecDev &sp, const DomainPlan &pl, int cap) {
  DomainArgs a = a0;
  for (int c = 0; c < pl.n_colours; ++c) {
    a.patch_begin = pl.colour_start[c];
    const int n = pl.colour_start[c + 1] - pl.colour_start[c];
    solid_patch_kernel<POLE, MODE_FORCE, false, false>
        <<<std::min(n, cap), kThreads, solid_smem_bytes<POLE, MODE_FORCE, false, false>(), 0>>>(a, st, sp, n,
                                                                                           AnelArgs{});
  }
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

}  // namespace

extern "C" int axg_stiffness_assembled_noalloc(const axg_mesh_desc *d, const float *u_gvec, float *f_gvec) {
  if (!u_gvec || !f_gvec) return fail(nullptr, AXG_ERR_BAD_ARG, "u_gvec and f_gvec must not be NULL");
  int rc = validate_stiffness(d);
  if (rc) return rc;
  if ((rc = check_igloc(d->igloc_solid, 25 * (int64_t)d->nel_solid, d->nglob_solid, "igloc_solid"))) return rc;
  if (axg_device_count() < 1) return fail(nullptr, AXG_ERR_NO_DEVICE, "no CUDA device is visible");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoAllocDevice *nd = nullptr;
  if ((rc = noalloc_setup(&nd))) return rc;

  // plan and pack on the host (the same planner as axg_create)
  const int pole = d->src_type;
  const int64_t nel = d->nel_solid, nglob = d->nglob_solid;
  DomainPlan pl;
  std::string perr = plan_domain(d->igloc_solid, nel, nglob, 0, -1, std::vector<uint8_t>(), pl, false, solid_plan_ctas());
  if (!perr.empty()) return fail(nullptr, AXG_ERR_BAD_DESC, "solid plan: " + perr);
  const std::vector<int> slots = solid_slots(pole), aslots = axial_slots(pole);
  const int nt = (int)slots.size(), na = (int)aslots.size();
  const int bs = solid_block_stride(nt);
  std::vector<uint8_t> axial(nel, 0);
  for (int k = 0; k < d->naxel_solid; ++k) axial[d->ax_el_solid[k] - 1] = 1;
  int64_t nax = 0;
  for (int64_t e = 0; e < nel; ++e) nax += axial[e];

  // scratch layout; everything 256-byte aligned
  const size_t o_meta = 0;
  const size_t o_pts = align256(o_meta + pl.meta.size() * sizeof(PatchMeta));
  const size_t o_metric = align256(o_pts + pl.pt_words.size() * sizeof(uint32_t));
  const size_t o_m0 = align256(o_metric + (size_t)nel * bs * sizeof(float));
  const size_t o_u = align256(o_m0 + (size_t)nax * na * 5 * sizeof(float));
  const size_t o_f = align256(o_u + (size_t)nglob * 3 * sizeof(float));
  const size_t o_ctl = align256(o_f + (size_t)nglob * 3 * sizeof(float));
  const size_t total = align256(o_ctl + 4 * sizeof(int32_t)) + 256;  // + tail pad
  if (total > kNoAllocScratchBytes)
    return fail(nullptr, AXG_ERR_BAD_ARG,
                fmt("mesh needs %zu bytes of device scratch; the no-allocation entry point holds at most %zu "
                    "bytes (%d elements of %d metric arrays need about %zu)",
                    total, kNoAllocScratchBytes, (int)nel, nt, (size_t)nel * bs * 4));

  std::vector<float> metric((size_t)nel * bs, 0.f), m0;
  m0.reserve((size_t)nax * na * 5);
  int32_t axcount = 0;
  for (int64_t s = 0; s < nel; ++s) {
    const int64_t e = pl.elem_order[s];
    float *blk = metric.data() + (size_t)s * bs;
    for (int t = 0; t < nt; ++t) std::memcpy(blk + 25 * t, d->m_solid[slots[t]] + 25 * e, 25 * sizeof(float));
    int32_t info = 0;
    if (axial[e]) {
      info = ++axcount;
      for (int q = 0; q < na; ++q)
        for (int jj = 0; jj < 5; ++jj) m0.push_back(d->m0_solid[aslots[q]][5 * e + jj]);
    }
    std::memcpy(blk + solid_idx_off(nt), &pl.elem_pts[25 * s], 25 * sizeof(uint16_t));
    std::memcpy(blk + solid_info_off(nt), &info, sizeof(int32_t));
  }

  unsigned char *base = nd->base;
  auto put = [&](size_t off, const void *src, size_t bytes) -> int {
    if (bytes == 0) return AXG_OK;
    cudaError_t e = cudaMemcpy(base + off, src, bytes, cudaMemcpyHostToDevice);
    return e == cudaSuccess ? AXG_OK : cuda_fail(nullptr, e, "cudaMemcpy to the no-allocation scratch");
  };
  const int32_t zeros[4] = {0, 0, 0, 0};  // the control words must start at zero on every call
  if ((rc = put(o_meta, pl.meta.data(), pl.meta.size() * sizeof(PatchMeta))) ||
      (rc = put(o_pts, pl.pt_words.data(), pl.pt_words.size() * sizeof(uint32_t))) ||
      (rc = put(o_metric, metric.data(), metric.size() * sizeof(float))) ||
      (rc = put(o_m0, m0.data(), m0.size() * sizeof(float))) ||
      (rc = put(o_u, u_gvec, (size_t)nglob * 3 * sizeof(float))) || (rc = put(o_ctl, zeros, sizeof zeros)))
    return rc;
  // the array keeps the previous call's force: a global point no element
  // refers to must read zero, not that value (cudaMemset allocates nothing)
  cudaError_t ez = cudaMemset(base + o_f, 0, (size_t)nglob * 3 * sizeof(float));
  if (ez != cudaSuccess) return cuda_fail(nullptr, ez, "cudaMemset of the no-allocation scratch");

  DomainArgs a{};
  a.meta = reinterpret_cast<const PatchMeta *>(base + o_meta);
  a.pts = reinterpret_cast<const uint32_t *>(base + o_pts);
  a.metric = reinterpret_cast<const float *>(base + o_metric);
  a.m0 = reinterpret_cast<const float *>(base + o_m0);
  a.n_patches = pl.n_patches;
  a.n_pts = pl.total_pts;
  a.n_elem = nel;
  a.n_m0 = (int64_t)m0.size();
  StateArgs st{};
  float *u = reinterpret_cast<float *>(base + o_u), *f = reinterpret_cast<float *>(base + o_f);
  for (int c = 0; c < 3; ++c) {
    st.u[c] = u + nglob * c;
    st.f[c] = f + nglob * c;
  }
  int32_t *ctl = reinterpret_cast<int32_t *>(base + o_ctl);
  st.iter = ctl;
  st.blowup = ctl + 1;
  st.err = ctl + 2;
  st.nglob = nglob;
  st.niter = 1;
  SpecDev sp{};
  for (int k = 0; k < 25; ++k) {
    sp.g1[k] = d->G1[k];
    sp.g2[k] = d->G2[k];
  }
  for (int k = 0; k < 5; ++k) sp.g0[k] = d->G0[k];
  if (pole == AXG_MONOPOLE) noalloc_launch<POLE_MONO>(a, st, sp, pl, nd->grid_cap[0]);
  else if (pole == AXG_DIPOLE) noalloc_launch<POLE_DI>(a, st, sp, pl, nd->grid_cap[1]);
  else noalloc_launch<POLE_QUAD>(a, st, sp, pl, nd->grid_cap[2]);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "no-allocation kernel launch");
  int32_t ctl_h[4];
  e = cudaMemcpy(f_gvec, f, (size_t)nglob * 3 * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(ctl_h, ctl, sizeof ctl_h, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMemcpy from the no-allocation scratch");
  if (ctl_h[2] != 0) return fail(nullptr, AXG_ERR_TIMEOUT, "a bounded device wait on a bulk copy gave up");
  if (pole == AXG_MONOPOLE) std::memset(f_gvec + nglob, 0, (size_t)nglob * sizeof(float));  // unused phi
  return AXG_OK;
}

namespace {
// Reads (out) or writes (in) one attenuation state field in the reference's
// layouts: memory_var_cg4(1:4,6,n_sls,nel_solid), src_tr_tm1_glob_cg4(1:4,
// nel_solid), src_dev_tm1_glob_cg4(1:4,6,nel_solid).
int anel_state_io(axg_handle *h, int field, float *out, const float *in) {
  if (field != AXG_FIELD_MEMVAR && field != AXG_FIELD_ATT_SRC_TR && field != AXG_FIELD_ATT_SRC_DEV)
    return fail(h, AXG_ERR_BAD_ARG, fmt("field %d not available", field));
  if (!h->anel && !h->anel_full)
    return fail(h, AXG_ERR_BAD_ARG, "the handle was created without attenuation (anel_true = 0)");
  const int64_t nel = h->nel_s, stride = h->an.state_stride;
  const int nsls = h->nsls;
  const int np = h->anel_full ? 25 : 4;  // points per element with memory variables
  int off = 0, len = 6 * np * nsls;  // floats per element of this field, and where they start in the state
  if (field == AXG_FIELD_ATT_SRC_TR) off = 6 * np * nsls, len = np;
  if (field == AXG_FIELD_ATT_SRC_DEV) off = 6 * np * nsls + np, len = 6 * np;
  std::vector<float> st((size_t)nel * stride);
  CK(cudaMemcpyAsync(st.data(), h->an.state, st.size() * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int64_t e = 0; e < nel; ++e) {
    float *blk = st.data() + (size_t)h->slot_of_elem_s[e] * stride + off;
    if (out) std::memcpy(out + (size_t)e * len, blk, len * sizeof(float));
    else std::memcpy(blk, in + (size_t)e * len, len * sizeof(float));
  }
  if (in) {
    CK(cudaMemcpyAsync(h->an.state, st.data(), st.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  return AXG_OK;
}
}  // namespace

// ============================================================== C-ABI

extern "C" {

const char *axg_version(void) { return "axisem_gb300 1 (sm_103a, patch-coloured assembly)"; }

int axg_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int axg_create(const axg_mesh_desc *d, axg_handle **out) { return axg_create_tuned(d, 0, -1, out); }

int axg_create_sharing(axg_handle *mesh_of, const axg_mesh_desc *d, axg_handle **out) {
  if (!out) return fail(nullptr, AXG_ERR_BAD_ARG, "out is NULL");
  *out = nullptr;
  if (!mesh_of) return fail(nullptr, AXG_ERR_BAD_ARG, "mesh_of is NULL");
  int rc = validate(d);
  if (rc) return rc;
  axg_handle *h = new axg_handle();
  rc = create_impl(h, d, mesh_of);
  if (rc) {
    g_create_error = h->err;
    release(h);
    delete h;
    return rc;
  }
  *out = h;
  return AXG_OK;
}

int axg_create_tuned(const axg_mesh_desc *d, int32_t patch_elems, int32_t growth, axg_handle **out) {
  if (!out) return fail(nullptr, AXG_ERR_BAD_ARG, "out is NULL");
  *out = nullptr;
  if (patch_elems < 0 || patch_elems > kMaxPatchElems)
    return fail(nullptr, AXG_ERR_BAD_ARG, fmt("patch_elems %d outside 0..%d", patch_elems, kMaxPatchElems));
  if (growth < -1 || growth > kGrowLayered) return fail(nullptr, AXG_ERR_BAD_ARG, "growth must be -1, 0 or 1");
  int rc = validate(d);
  if (rc) return rc;
  if (axg_device_count() < 1) return fail(nullptr, AXG_ERR_NO_DEVICE, "no CUDA device is visible");
  axg_handle *h = new axg_handle();
  h->patch_elems = patch_elems;
  h->growth = growth;
  rc = create_impl(h, d);
  if (rc) {
    g_create_error = h->err;
    release(h);
    delete h;
    return rc;
  }
  *out = h;
  return AXG_OK;
}

int axg_reset(axg_handle *h) {
  if (!h) return fail(nullptr, AXG_ERR_BAD_ARG, "handle is NULL");
  for (int c = 0; c < 3; ++c) {
    if (h->su[c]) CK(cudaMemsetAsync(h->su[c], 0, h->nglob_s * sizeof(float), h->stream));
    if (h->sv[c]) CK(cudaMemsetAsync(h->sv[c], 0, h->nglob_s * sizeof(float), h->stream));
    if (h->sa[c]) CK(cudaMemsetAsync(h->sa[c], 0, h->nglob_s * sizeof(float), h->stream));
    if (h->sf[c]) CK(cudaMemsetAsync(h->sf[c], 0, h->nglob_s * sizeof(float), h->stream));
  }
  if (h->nel_f > 0) {
    CK(cudaMemsetAsync(h->fu, 0, h->nglob_f * sizeof(float), h->stream));
    CK(cudaMemsetAsync(h->fv, 0, h->nglob_f * sizeof(float), h->stream));
    CK(cudaMemsetAsync(h->fa, 0, h->nglob_f * sizeof(float), h->stream));
    CK(cudaMemsetAsync(h->ff, 0, h->nglob_f * sizeof(float), h->stream));
  }
  // checkpoints restart with the run
  if (h->copy_stream) CK(cudaStreamSynchronize(h->copy_stream));
  if (int rc = checkpoint_progress(h)) return rc;
  h->ckpt.queued = h->ckpt.done = 0;
  // the iter-0 seismogram sample (dump_stuff(0,...)) is the zero wavefield
  CK(cudaMemsetAsync(h->rec, 0, (size_t)h->nseismo * 3 * std::max(h->num_rec, 1) * sizeof(float), h->stream));
  CK(cudaMemsetAsync(h->iter, 0, 4 * sizeof(int32_t), h->stream));
  if (h->anel || h->anel_full)
    CK(cudaMemsetAsync(h->an.state, 0, (size_t)h->nel_s * h->an.state_stride * sizeof(float), h->stream));
  for (float *p : {h->cu_s[0], h->cu_s[1], h->cu_s[2], h->cv_s[0], h->cv_s[1], h->cv_s[2], h->cu_f, h->cv_f})
    if (p) CK(cudaMemsetAsync(p, 0, (p == h->cu_f || p == h->cv_f ? h->nglob_f : h->nglob_s) * sizeof(float), h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return AXG_OK;
}

int axg_run(axg_handle *h, int32_t first_iter, int32_t n_iter) {
  if (!h) return fail(nullptr, AXG_ERR_BAD_ARG, "handle is NULL");
  if (n_iter < 0 || first_iter < 1 || (int64_t)first_iter + n_iter - 1 > h->niter)
    return fail(h, AXG_ERR_BAD_ARG, fmt("iterations %d..%d outside 1..niter=%d", first_iter, first_iter + n_iter - 1,
                                        h->niter));
  if (n_iter == 0) return AXG_OK;
  if (h->dump.type || h->ckpt.check_it > 0) {  // runs that dump or checkpoint: the asynchronous path
    int rc = axg_run_async(h, first_iter, n_iter);
    return rc ? rc : axg_wait(h);
  }
  CK(cudaMemcpyAsync(h->iter, &first_iter, sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  CK(refresh_predicted(h, h->stream));
  int32_t done = 0;
  while (done < n_iter) {
    const int k = std::min<int32_t>(h->steps_per_graph, n_iter - done);
    if (k == h->steps_per_graph) {
      const int rc = launch_graph(h, k, h->graph, h->graph_steps);
      if (rc) return rc;
    } else {
      for (int s = 0; s < k; ++s) enqueue_step(h, h->stream);
      CK(cudaGetLastError());
    }
    done += k;
    int32_t flags[2] = {0, 0};
    CK(cudaMemcpyAsync(flags, h->blowup, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    const int32_t bl = flags[0];
    if (flags[1] != 0)
      return fail(h, AXG_ERR_TIMEOUT, "a bounded device wait on a bulk copy gave up");
    if (bl != 0)
      return fail(h, AXG_ERR_BLOWUP,
                  fmt("displacements blew up: |disp(1,1,:,:)| > 10 |magnitude| at time step %d", bl + 1));
  }
  return AXG_OK;
}

}  // extern "C"

namespace {
// reads the device flags after the handle's queued work completed
int check_flags(axg_handle *h) {
  int32_t flags[2] = {0, 0};
  CK(cudaMemcpyAsync(flags, h->blowup, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (flags[1] != 0) return fail(h, AXG_ERR_TIMEOUT, "a bounded device wait on a bulk copy gave up");
  if (flags[0] != 0)
    return fail(h, AXG_ERR_BLOWUP,
                fmt("displacements blew up: |disp(1,1,:,:)| > 10 |magnitude| at time step %d", flags[0] + 1));
  return AXG_OK;
}

// The gvec I/O (axg_upload_gvec_disp / axg_download_gvec_force) is in the
// reference's point numbering, the handle's arrays in the plan's.  The host
// copies go through a staging buffer in chunks of points on a copy stream;
// a permutation kernel on the handle's stream moves each chunk as soon as it
// has landed (uploads) or before it leaves (downloads), so that copies and
// permutations overlap.  (Letting the permutation kernel read and write a
// pinned host buffer directly over the CPU-GPU link was slower on GB300:
// 3.21 against 2.95 ms for a 1024 x 1024 quadrupole step, the copy engines
// moving ~200 GB/s each way; 8 or 16 chunks gained nothing over 4.)
constexpr int kGvecChunks = 4;

// a step counter set on the stream, without a host synchronisation
__global__ void set_counter_kernel(int32_t *ctr, int32_t v) { *ctr = v; }

static_assert(sizeof(axg_handle::ev_io) / sizeof(cudaEvent_t) == kGvecChunks + 1, "one event per chunk + one");

// u[c][new_of_old[g]] = stage[c][g], g in [a, b)
__global__ void gvec_to_internal_kernel(const float *__restrict__ stage, const int32_t *__restrict__ new_of_old,
                                        int64_t n, int64_t a, int64_t b, float *u0, float *u1, float *u2) {
  for (int64_t g = a + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < b; g += (int64_t)gridDim.x * blockDim.x) {
    const int32_t t = new_of_old[g];
    if (u0) u0[t] = stage[g];
    if (u1) u1[t] = stage[n + g];
    if (u2) u2[t] = stage[2 * n + g];
  }
}

// stage[c][g] = f[c][new_of_old[g]], g in [a, b)
__global__ void gvec_from_internal_kernel(const float *__restrict__ f0, const float *__restrict__ f1,
                                          const float *__restrict__ f2, const int32_t *__restrict__ new_of_old,
                                          int64_t n, int64_t a, int64_t b, float *stage) {
  for (int64_t g = a + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < b; g += (int64_t)gridDim.x * blockDim.x) {
    const int32_t t = new_of_old[g];
    if (f0) stage[g] = f0[t];
    if (f1) stage[n + g] = f1[t];
    if (f2) stage[2 * n + g] = f2[t];
  }
}

unsigned gvec_grid(const axg_handle *h, int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 8 * (int64_t)h->num_sms));
}

// the permutation, staging buffer, copy stream and events, on first use
int gvec_io_prepare(axg_handle *h) {
  if (h->gvec_perm) return AXG_OK;
  int rc;
  if ((rc = upload(h, &h->gvec_perm, h->ps.new_of_old))) return rc;
  if ((rc = dalloc(h, &h->gvec_stage, 3 * (size_t)h->nglob_s))) return rc;
  if (!h->copy_stream) CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
  for (cudaEvent_t &e : h->ev_io) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return AXG_OK;
}

// ---- kernel wavefield dumps

// the fields of a dump type for one domain, with the reference's names
std::vector<std::string> dump_fields(int type, int pole, bool fluid) {
  const bool nm = pole != AXG_MONOPOLE;
  const std::string dom = fluid ? "_flu" : "_sol";
  std::vector<std::string> f;
  auto strain = [&]() {
    for (const char *n : {"strain_dsus", "strain_dsuz", "strain_dpup", "straintrace"}) f.push_back(n + dom);
    if (nm)
      for (const char *n : {"strain_dsup", "strain_dzup"}) f.push_back(n + dom);
  };
  auto vec = [&](const std::string &v) {
    f.push_back(v + dom + "_s");
    if (nm) f.push_back(v + dom + "_p");
    f.push_back(v + dom + "_z");
  };
  if (type == AXG_DUMP_STRAIN_ONLY || type == AXG_DUMP_FULLFIELDS) strain();
  if (type == AXG_DUMP_DISPL_ONLY) vec("disp");
  if (type == AXG_DUMP_DISPL_VELO) {
    if (fluid) {
      f.push_back("chi_flu");
      f.push_back("dchi_flu");
    } else {
      vec("disp");
      vec("velo");
    }
  }
  if (type == AXG_DUMP_FULLFIELDS) vec("velo");
  return f;
}

template <int POLE>
void launch_dump_pole(axg_handle *h, float *slot) {
  const Dump &dp = h->dump;
  const unsigned ws = kThreads / 32;
  DumpArgs a{};
  a.type = dp.type;
  a.ibeg = dp.ibeg;
  a.iend = dp.iend;
  a.jbeg = dp.jbeg;
  a.jend = dp.jend;
  a.gidx = dp.gidx_s;
  a.axial = dp.ax_s;
  for (int k = 0; k < 5; ++k) a.pw[k] = dp.pw_s[k];
  for (int c = 0; c < 3; ++c) {
    a.u[c] = h->su[c];
    a.v[c] = h->sv[c];
  }
  a.out = slot;
  a.nel = h->nel_s;
  a.nglob = h->nglob_s;
  a.kwf = dp.kwf ? dp.kwf_s : nullptr;
  a.npt = dp.npt_s;
  a.nsrcel = 0;
  if (dp.src_mask)
    for (int32_t e : h->ielsrc) a.srcel[a.nsrcel++] = e;
  const unsigned gs = (unsigned)std::min<int64_t>((h->nel_s + ws - 1) / ws, 16 * (int64_t)h->num_sms);
  wavefield_dump_kernel<POLE, false><<<gs, kThreads, 0, h->stream>>>(a, h->spec);
  if (h->nel_f > 0 && dp.nf > 0) {
    a.gidx = dp.gidx_f;
    a.axial = dp.ax_f;
    for (int k = 0; k < 5; ++k) a.pw[k] = dp.pw_f[k];
    a.inv_rho = dp.inv_rho;
    a.u[0] = h->fu;
    a.v[0] = h->fv;
    a.u[1] = a.u[2] = a.v[1] = a.v[2] = nullptr;
    a.out = slot + (dp.kwf ? (int64_t)dp.ns * dp.npt_s : (int64_t)dp.ns * h->nel_s * dp.np);
    a.nel = h->nel_f;
    a.nglob = h->nglob_f;
    a.kwf = dp.kwf ? dp.kwf_f : nullptr;
    a.npt = dp.npt_f;
    const unsigned gf = (unsigned)std::min<int64_t>((h->nel_f + ws - 1) / ws, 16 * (int64_t)h->num_sms);
    wavefield_dump_kernel<POLE, true><<<gf, kThreads, 0, h->stream>>>(a, h->spec);
  }
}

// snapshot `idx` from the state at the end of the steps queued so far: the
// kernels write one of two device slots, the copy stream moves it to the
// host buffer while the next steps run
int enqueue_dump(axg_handle *h, int64_t idx) {
  Dump &dp = h->dump;
  const int k = (int)(idx & 1);
  CK(cudaStreamWaitEvent(h->stream, dp.ev_copy[k], 0));  // the slot's previous snapshot has left
  if (h->pole == AXG_MONOPOLE) launch_dump_pole<POLE_MONO>(h, dp.slot[k]);
  else if (h->pole == AXG_DIPOLE) launch_dump_pole<POLE_DI>(h, dp.slot[k]);
  else launch_dump_pole<POLE_QUAD>(h, dp.slot[k]);
  CK(cudaGetLastError());
  CK(cudaEventRecord(dp.ev_dump[k], h->stream));
  CK(cudaStreamWaitEvent(h->copy_stream, dp.ev_dump[k], 0));
  CK(cudaMemcpyAsync(dp.out + idx * dp.floats, dp.slot[k], dp.floats * sizeof(float), cudaMemcpyDeviceToHost,
                     h->copy_stream));
  CK(cudaEventRecord(dp.ev_copy[k], h->copy_stream));
  return AXG_OK;
}

// seismogram checkpoint after iteration `last_it` (queued on the handle's
// stream): the samples the steps up to the latest multiple of check_it have
// recorded -- sample 0 is iteration 0, then one every seis_it steps -- are
// final; the ones not yet copied go to the caller's buffer in one strided copy
// of every (component, receiver) column, on the copy stream
int enqueue_checkpoint(axg_handle *h, int32_t last_it) {
  auto &ck = h->ckpt;
  const int32_t c = last_it / ck.check_it * ck.check_it;
  if (c <= 0 || h->num_rec <= 0) return AXG_OK;
  const int32_t s1 = std::min<int32_t>(c / std::max(h->seis_it, 1) + 1, std::min(ck.cap, h->nseismo));
  if (s1 <= ck.queued) return AXG_OK;
  if (!h->copy_stream) CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
  cudaEvent_t ev;
  if (ck.free_events.empty()) {
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  } else {
    ev = ck.free_events.back();
    ck.free_events.pop_back();
  }
  CK(cudaEventRecord(ev, h->stream));
  CK(cudaStreamWaitEvent(h->copy_stream, ev, 0));
  const int32_t s0 = ck.queued;
  CK(cudaMemcpy2DAsync(ck.out + s0, (size_t)ck.cap * sizeof(float), h->rec + s0, (size_t)h->nseismo * sizeof(float),
                       (size_t)(s1 - s0) * sizeof(float), (size_t)3 * h->num_rec, cudaMemcpyDeviceToHost,
                       h->copy_stream));
  CK(cudaEventRecord(ev, h->copy_stream));
  ck.inflight.emplace_back(ev, s1);
  ck.queued = s1;
  return AXG_OK;
}

// completed checkpoint copies (non-blocking)
int checkpoint_progress(axg_handle *h) {
  auto &ck = h->ckpt;
  while (!ck.inflight.empty()) {
    const cudaError_t e = cudaEventQuery(ck.inflight.front().first);
    if (e == cudaErrorNotReady) {
      cudaGetLastError();
      break;
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "checkpoint copy");
    ck.done = ck.inflight.front().second;
    ck.free_events.push_back(ck.inflight.front().first);
    ck.inflight.pop_front();
  }
  return AXG_OK;
}
}  // namespace

extern "C" {

int axg_run_async(axg_handle *h, int32_t first_iter, int32_t n_iter) {
  if (!h) return fail(nullptr, AXG_ERR_BAD_ARG, "handle is NULL");
  if (n_iter < 0 || first_iter < 1 || (int64_t)first_iter + n_iter - 1 > h->niter)
    return fail(h, AXG_ERR_BAD_ARG, fmt("iterations %d..%d outside 1..niter=%d", first_iter, first_iter + n_iter - 1,
                                        h->niter));
  if (n_iter == 0) return AXG_OK;
  const Dump &dp = h->dump;
  if (dp.type) {
    const int64_t last = ((int64_t)first_iter + n_iter - 1) / dp.strain_it - 1;  // last snapshot of the run
    if (last >= dp.capacity)
      return fail(h, AXG_ERR_BAD_ARG, fmt("snapshot %lld of the run is beyond the dump buffer's capacity %lld",
                                          (long long)last, (long long)dp.capacity));
  }
  // the kernels of a step after a blow-up return at once, so all steps can
  // be queued without a check in between
  CK(cudaMemcpyAsync(h->iter, &first_iter, sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  CK(refresh_predicted(h, h->stream));
  for (int32_t done = 0; done < n_iter;) {
    const int32_t it = first_iter + done;
    int k = std::min<int32_t>(h->steps_per_graph, n_iter - done);
    if (dp.type) k = std::min<int32_t>(k, dp.strain_it - (it - 1) % dp.strain_it);  // up to the next dump
    if (k == h->steps_per_graph) {
      const int rc = launch_graph(h, k, h->graph, h->graph_steps);
      if (rc) return rc;
    } else if (dp.type && k == dp.strain_it) {
      const int rc = launch_graph(h, k, h->graph_dump, h->graph_dump_steps);
      if (rc) return rc;
    } else {
      for (int q = 0; q < k; ++q) enqueue_step(h, h->stream);
      CK(cudaGetLastError());
    }
    done += k;
    const int32_t last_it = first_iter + done - 1;
    if (dp.type && last_it % dp.strain_it == 0) {
      int rc = enqueue_dump(h, last_it / dp.strain_it - 1);
      if (rc) return rc;
    }
    if (h->ckpt.check_it > 0) {
      int rc = enqueue_checkpoint(h, last_it);
      if (rc) return rc;
    }
  }
  if (dp.type)  // the run is complete once its snapshots are in the host buffer
    for (int k = 0; k < 2; ++k) CK(cudaStreamWaitEvent(h->stream, dp.ev_copy[k], 0));
  if (!h->ckpt.inflight.empty())  // and its checkpoint copies
    CK(cudaStreamWaitEvent(h->stream, h->ckpt.inflight.back().first, 0));
  CK(cudaEventRecord(h->ev_done, h->stream));
  h->pending = true;
  return AXG_OK;
}

int axg_poll(axg_handle *h, int32_t *done) {
  if (!h || !done) return fail(h, AXG_ERR_BAD_ARG, "NULL argument");
  *done = 1;
  if (!h->pending) return AXG_OK;
  const cudaError_t e = cudaEventQuery(h->ev_done);
  if (e == cudaErrorNotReady) {
    *done = 0;
    return AXG_OK;
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaEventQuery");
  h->pending = false;
  return check_flags(h);
}

int axg_wait(axg_handle *h) {
  if (!h) return fail(nullptr, AXG_ERR_BAD_ARG, "handle is NULL");
  CK(cudaStreamSynchronize(h->stream));
  h->pending = false;
  int rc = checkpoint_progress(h);
  return rc ? rc : check_flags(h);
}

int axg_set_seismogram_checkpoint(axg_handle *h, int32_t check_it, float *out, int32_t nseismo_cap) {
  if (!h) return fail(nullptr, AXG_ERR_BAD_ARG, "handle is NULL");
  if (h->pending) return fail(h, AXG_ERR_BAD_ARG, "the handle has queued steps");
  if (check_it < 0) return fail(h, AXG_ERR_BAD_ARG, "check_it must be >= 0");
  if (check_it > 0 && (!out || nseismo_cap < 1)) return fail(h, AXG_ERR_BAD_ARG, "out and nseismo_cap are required");
  CK(cudaStreamSynchronize(h->stream));
  if (h->copy_stream) CK(cudaStreamSynchronize(h->copy_stream));
  int rc = checkpoint_progress(h);
  if (rc) return rc;
  auto &ck = h->ckpt;
  ck.check_it = check_it;
  ck.out = out;
  ck.cap = nseismo_cap;
  ck.queued = ck.done = 0;
  return AXG_OK;
}

int axg_seismogram_checkpoint_samples(axg_handle *h, int32_t *n_samples) {
  if (!h || !n_samples) return fail(h, AXG_ERR_BAD_ARG, "NULL argument");
  int rc = checkpoint_progress(h);
  if (rc) return rc;
  *n_samples = h->ckpt.done;
  return AXG_OK;
}

int axg_get_receivers(axg_handle *h, float *out, int32_t cap, int32_t *nseismo_out) {
  if (!h || !out) return fail(h, AXG_ERR_BAD_ARG, "NULL argument");
  if (cap < h->nseismo) return fail(h, AXG_ERR_BAD_ARG, fmt("nseismo_cap %d < nseismo %d", cap, h->nseismo));
  std::vector<float> buf((size_t)h->nseismo * 3 * std::max(h->num_rec, 1));
  CK(cudaMemcpyAsync(buf.data(), h->rec, buf.size() * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  int32_t it = 0;
  CK(cudaMemcpyAsync(&it, h->iter, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int r = 0; r < h->num_rec; ++r)
    for (int c = 0; c < 3; ++c)
      for (int s = 0; s < h->nseismo; ++s)
        out[s + (int64_t)cap * (c + 3 * (int64_t)r)] = buf[s + (int64_t)h->nseismo * (c + 3 * (int64_t)r)];
  // samples written: iter 0 plus every seis_it steps completed
  const int32_t last = it > 0 ? it - 1 : 0;
  if (nseismo_out) *nseismo_out = std::min(h->nseismo, last / h->seis_it + 1);
  return AXG_OK;
}

int axg_get_state(axg_handle *h, int32_t field, float *out) {
  if (!h || !out) return fail(h, AXG_ERR_BAD_ARG, "NULL argument");
  if (field >= AXG_FIELD_MEMVAR && field <= AXG_FIELD_ATT_SRC_DEV) return anel_state_io(h, field, out, nullptr);
  float *p[3] = {};
  int nc;
  int64_t ng;
  bool fluid;
  int rc = state_ptrs(h, field, p, &nc, &ng, &fluid);
  if (rc) return rc;
  const std::vector<int32_t> &ig = fluid ? h->igloc_f : h->igloc_s;
  const int64_t cs = (int64_t)ig.size();
  std::vector<float> g(ng);
  for (int c = 0; c < nc; ++c) {
    if (!p[c]) {
      std::fill(out + cs * c, out + cs * (c + 1), 0.f);
      continue;
    }
    CK(cudaMemcpyAsync(g.data(), p[c], ng * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int64_t q = 0; q < cs; ++q) out[q + cs * c] = g[ig[q] - 1];
  }
  return AXG_OK;
}

int axg_set_state(axg_handle *h, int32_t field, const float *in) {
  if (!h || !in) return fail(h, AXG_ERR_BAD_ARG, "NULL argument");
  if (field >= AXG_FIELD_MEMVAR && field <= AXG_FIELD_ATT_SRC_DEV) return anel_state_io(h, field, nullptr, in);
  float *p[3] = {};
  int nc;
  int64_t ng;
  bool fluid;
  int rc = state_ptrs(h, field, p, &nc, &ng, &fluid);
  if (rc) return rc;
  const std::vector<int32_t> &ig = fluid ? h->igloc_f : h->igloc_s;
  const int64_t cs = (int64_t)ig.size();
  for (int c = 0; c < nc; ++c) {
    if (!p[c]) continue;
    std::vector<float> g = per_point(in + cs * c, ig, ng);
    CK(cudaMemcpyAsync(p[c], g.data(), ng * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  return AXG_OK;
}

int axg_upload_gvec_disp(axg_handle *h, const float *u) {
  if (!h || !u) return fail(h, AXG_ERR_BAD_ARG, "NULL argument");
  int rc = gvec_io_prepare(h);
  if (rc) return rc;
  const int64_t n = h->nglob_s;
  // the staging buffer is free once the work queued so far has run
  CK(cudaEventRecord(h->ev_io[kGvecChunks], h->stream));
  CK(cudaStreamWaitEvent(h->copy_stream, h->ev_io[kGvecChunks], 0));
  for (int k = 0; k < kGvecChunks; ++k) {
    const int64_t a = n * k / kGvecChunks, b = n * (k + 1) / kGvecChunks;
    for (int c = 0; c < 3; ++c)
      if (h->su[c])
        CK(cudaMemcpyAsync(h->gvec_stage + n * c + a, u + n * c + a, (b - a) * sizeof(float),
                           cudaMemcpyHostToDevice, h->copy_stream));
    CK(cudaEventRecord(h->ev_io[k], h->copy_stream));
    CK(cudaStreamWaitEvent(h->stream, h->ev_io[k], 0));
    gvec_to_internal_kernel<<<gvec_grid(h, b - a), 256, 0, h->stream>>>(h->gvec_stage, h->gvec_perm, n, a, b,
                                                                         h->su[0], h->su[1], h->su[2]);
    CK(cudaGetLastError());
  }
  return AXG_OK;
}

int axg_download_gvec_force(axg_handle *h, float *f) {
  if (!h || !f) return fail(h, AXG_ERR_BAD_ARG, "NULL argument");
  int rc = gvec_io_prepare(h);
  if (rc) return rc;
  const int64_t n = h->nglob_s;
  for (int k = 0; k < kGvecChunks; ++k) {
    const int64_t a = n * k / kGvecChunks, b = n * (k + 1) / kGvecChunks;
    gvec_from_internal_kernel<<<gvec_grid(h, b - a), 256, 0, h->stream>>>(h->sf[0], h->sf[1], h->sf[2],
                                                                           h->gvec_perm, n, a, b, h->gvec_stage);
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->ev_io[k], h->stream));
    CK(cudaStreamWaitEvent(h->copy_stream, h->ev_io[k], 0));
    for (int c = 0; c < 3; ++c)
      if (h->sf[c])
        CK(cudaMemcpyAsync(f + n * c + a, h->gvec_stage + n * c + a, (b - a) * sizeof(float),
                           cudaMemcpyDeviceToHost, h->copy_stream));
  }
  for (int c = 0; c < 3; ++c)
    if (!h->sf[c]) std::memset(f + n * c, 0, n * sizeof(float));
  CK(cudaStreamSynchronize(h->copy_stream));
  return AXG_OK;
}

int axg_stiffness_assembled_device(axg_handle *h, void *stream) {
  if (!h) return fail(nullptr, AXG_ERR_BAD_ARG, "handle is NULL");
  cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
  enqueue_force(h, s);
  CK(cudaGetLastError());
  return AXG_OK;
}

int axg_stiffness_assembled(axg_handle *h, const float *u, float *f) {
  if (!h || !u || !f) return fail(h, AXG_ERR_BAD_ARG, "NULL argument");
  int rc = axg_upload_gvec_disp(h, u);
  if (rc) return rc;
  enqueue_force(h, h->stream);
  CK(cudaGetLastError());
  return axg_download_gvec_force(h, f);
}

int axg_set_tuning(axg_handle *h, int32_t patch_elems, int32_t steps_per_graph) {
  if (!h) return fail(nullptr, AXG_ERR_BAD_ARG, "handle is NULL");
  if (steps_per_graph < 0 || steps_per_graph > 4096) return fail(h, AXG_ERR_BAD_ARG, "steps_per_graph out of range");
  if (patch_elems != 0 && patch_elems != h->ps.patch_elems)
    return fail(h, AXG_ERR_UNSUPPORTED, "the patch shape is fixed at creation (axg_create_tuned)");
  if (steps_per_graph > 0 && steps_per_graph != h->steps_per_graph) {
    h->steps_per_graph = steps_per_graph;
    drop_graphs(h);
  }
  return AXG_OK;
}

int axg_autotune(axg_handle *h, int32_t *chosen) {
  if (!h) return fail(nullptr, AXG_ERR_BAD_ARG, "handle is NULL");
  if (h->pending) return fail(h, AXG_ERR_BAD_ARG, "the handle has queued steps");
  // every device array a step writes: saved, then restored
  std::vector<std::pair<void *, size_t>> st;
  auto add = [&](void *p, size_t bytes) {
    if (p && bytes) st.emplace_back(p, bytes);
  };
  const size_t gs = h->nglob_s * sizeof(float), gf = std::max<int64_t>(h->nglob_f, 0) * sizeof(float);
  for (int c = 0; c < 3; ++c) {
    add(h->su[c], gs), add(h->sv[c], gs), add(h->sa[c], gs), add(h->sf[c], gs);
    add(h->cu_s[c], gs), add(h->cv_s[c], gs);
  }
  add(h->fu, gf), add(h->fv, gf), add(h->fa, gf), add(h->ff, gf), add(h->cu_f, gf), add(h->cv_f, gf);
  if (h->anel || h->anel_full) add(h->an.state, (size_t)h->nel_s * h->an.state_stride * sizeof(float));
  add(h->rec, (size_t)h->nseismo * 3 * std::max(h->num_rec, 1) * sizeof(float));
  add(h->iter, 4 * sizeof(int32_t));
  size_t total = 0;
  for (auto &p : st) total += (p.second + 255) / 256 * 256;
  char *save = nullptr;
  CK(cudaMallocAsync((void **)&save, total, h->stream));
  // from here on errors are collected, so that the state is restored and the
  // scratch freed on every path
  cudaError_t ce = cudaSuccess;
  size_t off = 0;
  for (auto &p : st) {
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(save + off, p.first, p.second, cudaMemcpyDeviceToDevice, h->stream);
    off += (p.second + 255) / 256 * 256;
  }
  if (ce == cudaSuccess) ce = refresh_predicted(h, h->stream);
  int best = h->steps_per_graph, rc = ce == cudaSuccess ? AXG_OK : cuda_fail(h, ce, "axg_autotune: saving the state");
  float best_ms = 0.f;
  for (int k = 2; k <= 64 && rc == AXG_OK; k *= 2) {
    // one untimed launch, then `reps` launches of at least 256 steps in all;
    // the step counter restarts at 1 whenever the next launch would pass niter
    const int per_run = h->niter / k;  // launches from iteration 1 within niter
    if (per_run < 1) break;
    const int reps = std::max(1, 256 / k);
    cudaGraphExec_t g = nullptr;
    if ((rc = build_graph_into(h, k, &g))) break;
    float ms = 0.f;
    set_counter_kernel<<<1, 1, 0, h->stream>>>(h->iter, 1);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaGraphLaunch(g, h->stream);
    int in_run = 1;
    if (e == cudaSuccess) e = cudaEventRecord(h->ev0, h->stream);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) {
      if (in_run == per_run) {
        set_counter_kernel<<<1, 1, 0, h->stream>>>(h->iter, 1);
        e = cudaGetLastError();
        in_run = 0;
      }
      if (e == cudaSuccess) e = cudaGraphLaunch(g, h->stream);
      ++in_run;
    }
    if (e == cudaSuccess) e = cudaEventRecord(h->ev1, h->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(h->ev1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    cudaGraphExecDestroy(g);
    if (e != cudaSuccess) {
      rc = cuda_fail(h, e, "axg_autotune");
      break;
    }
    const float per_step = ms / (reps * k);
    if (best_ms == 0.f || per_step < best_ms) {
      best_ms = per_step;
      best = k;
    }
  }
  off = 0;
  ce = cudaSuccess;
  for (auto &p : st) {  // the solve's state as it was
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(p.first, save + off, p.second, cudaMemcpyDeviceToDevice, h->stream);
    off += (p.second + 255) / 256 * 256;
  }
  const cudaError_t fe = cudaFreeAsync(save, h->stream);
  if (ce == cudaSuccess) ce = fe;
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->stream);
  if (rc) return rc;
  if (ce != cudaSuccess) return cuda_fail(h, ce, "axg_autotune: restoring the state");
  if (best != h->steps_per_graph) {
    h->steps_per_graph = best;
    drop_graphs(h);
  }
  if (chosen) *chosen = best;
  return AXG_OK;
}

int axg_set_compensated(axg_handle *h, int32_t on) {
  if (!h) return fail(nullptr, AXG_ERR_BAD_ARG, "handle is NULL");
  if (on && !h->cu_s[0]) {
    // first use: zeroed compensation for every stored component
    int rc;
    const bool mono = h->pole == AXG_MONOPOLE;
    for (int c = 0; c < 3; ++c) {
      if (mono && c == 1) continue;
      if ((rc = dalloc(h, &h->cu_s[c], h->nglob_s)) || (rc = dalloc(h, &h->cv_s[c], h->nglob_s))) return rc;
      CK(cudaMemsetAsync(h->cu_s[c], 0, h->nglob_s * sizeof(float), h->stream));
      CK(cudaMemsetAsync(h->cv_s[c], 0, h->nglob_s * sizeof(float), h->stream));
    }
    if (h->nel_f > 0) {
      if ((rc = dalloc(h, &h->cu_f, h->nglob_f)) || (rc = dalloc(h, &h->cv_f, h->nglob_f))) return rc;
      CK(cudaMemsetAsync(h->cu_f, 0, h->nglob_f * sizeof(float), h->stream));
      CK(cudaMemsetAsync(h->cv_f, 0, h->nglob_f * sizeof(float), h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
  }
  h->kahan = on != 0;
  drop_graphs(h);
  return prepare_kernels(h);
}

int axg_symplectic_coefficients(int32_t scheme, double deltat, double *coefd, double *coefv, double *coeff,
                                int32_t *nstages) {
  if (!coefd || !coefv || !coeff || !nstages) return fail(nullptr, AXG_ERR_BAD_ARG, "NULL argument");
  std::vector<double> cd, cv;
  const int n = symplectic_coefficients(scheme, cd, cv);
  if (n == 0) return fail(nullptr, AXG_ERR_BAD_ARG, fmt("scheme %d is not a symplectic scheme", scheme));
  double acc = 0.0;
  for (int i = 0; i <= n; ++i) coefd[i] = cd[i] * deltat;  // coefd = coefd * deltat
  for (int i = 0; i < n; ++i) {
    coefv[i] = cv[i] * deltat;
    acc += coefd[i];
    coeff[i] = acc;  // coeff(i) = sum(coefd(1:i))
  }
  *nstages = n;
  return AXG_OK;
}

int axg_set_time_scheme(axg_handle *h, int32_t scheme, const float *stf_stages) {
  if (!h) return fail(nullptr, AXG_ERR_BAD_ARG, "handle is NULL");
  if (scheme == AXG_SCHEME_NEWMARK2) {
    h->scheme = 0;
    h->nstages = 0;
  } else {
    std::vector<double> cd, cv;
    const int n = symplectic_coefficients(scheme, cd, cv);
    if (n == 0) return fail(h, AXG_ERR_BAD_ARG, fmt("unknown time scheme %d", scheme));
    if (h->fluid_src || h->df.fsmask)
      return fail(h, AXG_ERR_UNSUPPORTED,
                  "symplectic schemes: a fluid source and a fluid free surface are not supported (the reference's "
                  "symplectic loop applies neither)");
    if (!stf_stages) return fail(h, AXG_ERR_BAD_ARG, "stf_stages is NULL");
    if (h->anel_full)
      return fail(h, AXG_ERR_UNSUPPORTED,
                  "symplectic schemes with attenuation at every GLL point (att_coarse_grained = 0) are not supported");
    if (h->anel) {  // per launch slot: the element's points and axis flag
      const int rc = upload_slot_points(h);
      if (rc) return rc;
    }
    h->sym_cd.resize(n + 1);
    h->sym_cv.resize(n);
    for (int i = 0; i <= n; ++i) h->sym_cd[i] = cd[i] * h->dt;
    for (int i = 0; i < n; ++i) h->sym_cv[i] = cv[i] * h->dt;
    std::vector<float> stf(stf_stages, stf_stages + (size_t)std::max(h->niter, 1) * n);
    int rc;
    if ((rc = upload(h, &h->stf_stages, stf))) return rc;
    h->scheme = scheme;
    h->nstages = n;
  }
  drop_graphs(h);
  int rc = prepare_kernels(h);
  if (rc) return rc;
  if (h->scheme) {
    h->kernels_per_step = (int64_t)h->nstages * (h->ps.n_colours + (h->nel_f > 0 ? 2 +
                          (h->to_fluid.n > 0) + (h->to_solid.n > 0) : 0)) + 2 + (h->anel ? 1 : 0);
  } else {
    h->kernels_per_step = h->ps.n_colours + 1 + (h->anel_full ? 1 : 0) +
                          (h->nel_f > 0 ? 2 + (h->to_fluid.n > 0) + (h->to_solid.n > 0) : 0);
  }
  return axg_reset(h);
}

int axg_get_info(axg_handle *h, axg_info *info) {
  if (!h || !info) return fail(h, AXG_ERR_BAD_ARG, "NULL argument");
  std::memset(info, 0, sizeof *info);
  info->n_patches_solid = h->ps.n_patches;
  info->n_patches_fluid = h->pf.n_patches;
  info->n_colours_solid = h->ps.n_colours;
  info->n_colours_fluid = h->pf.n_colours;
  info->max_subrounds_solid = h->ps.max_rounds;
  info->max_subrounds_fluid = h->pf.max_rounds;
  info->device_bytes = h->dev_bytes;
  info->kernels_per_step = h->kernels_per_step;
  info->kernels_per_force = h->kernels_per_force;
  info->patch_points_solid = 0;
  for (const PatchMeta &m : h->ps.meta) info->patch_points_solid += m.n_pts;
  info->patch_elems_solid = h->ps.patch_elems;
  info->growth_solid = h->ps.growth;
  info->patch_elems_fluid = h->pf.patch_elems;
  info->growth_fluid = h->pf.growth;
  info->steps_per_graph = h->steps_per_graph;
  info->mesh_bytes = h->mesh ? h->mesh->bytes : 0;
  info->ctas_per_sm_force = h->solid_ctas / std::max(h->num_sms, 1);
  info->ctas_per_sm_step = h->solid_ctas_step / std::max(h->num_sms, 1);
  return AXG_OK;
}

int axg_get_solid_colouring(axg_handle *h, int32_t *patch_of_elem, int32_t *colour_of_patch, int64_t cap) {
  if (!h || !patch_of_elem || !colour_of_patch) return fail(h, AXG_ERR_BAD_ARG, "NULL argument");
  if (cap < h->ps.n_patches) return fail(h, AXG_ERR_BAD_ARG, "n_patch_cap too small");
  std::memcpy(patch_of_elem, h->ps.patch_of_elem.data(), h->nel_s * sizeof(int32_t));
  std::memcpy(colour_of_patch, h->ps.colour_of_patch.data(), h->ps.n_patches * sizeof(int32_t));
  return AXG_OK;
}

int axg_plan_check(const axg_mesh_desc *d, int32_t patch_elems, int32_t growth, axg_info *info) {
  return axg_plan_check_ctas(d, patch_elems, growth, 0, info);
}

int axg_plan_check_ctas(const axg_mesh_desc *d, int32_t patch_elems, int32_t growth, int32_t ctas, axg_info *info) {
  if (!info) return fail(nullptr, AXG_ERR_BAD_ARG, "info is NULL");
  if (ctas < 0) return fail(nullptr, AXG_ERR_BAD_ARG, "ctas < 0");
  int rc = validate(d);
  if (rc) return rc;
  if ((rc = check_igloc(d->igloc_solid, 25 * (int64_t)d->nel_solid, d->nglob_solid, "igloc_solid"))) return rc;
  if (d->nel_fluid > 0 &&
      (rc = check_igloc(d->igloc_fluid, 25 * (int64_t)d->nel_fluid, d->nglob_fluid, "igloc_fluid")))
    return rc;
  std::vector<uint8_t> pre_s, pre_f;
  prepass_flags(d, pre_s, pre_f);
  std::memset(info, 0, sizeof *info);
  DomainPlan ps, pf;
  if (patch_elems < 0 || patch_elems > kMaxPatchElems) return fail(nullptr, AXG_ERR_BAD_ARG, "patch_elems out of range");
  if (growth < -1 || growth > kGrowLayered) return fail(nullptr, AXG_ERR_BAD_ARG, "growth must be -1, 0 or 1");
  std::string e = plan_domain(d->igloc_solid, d->nel_solid, d->nglob_solid, patch_elems, growth, pre_s, ps, true, ctas,
                              d->anel_true != 0 && d->att_coarse_grained != 0);
  if (e.empty()) e = validate_plan(d->igloc_solid, d->nel_solid, d->nglob_solid, pre_s, ps);
  if (!e.empty()) return fail(nullptr, AXG_ERR_BAD_DESC, "solid plan: " + e);
  if (d->nel_fluid > 0) {
    e = plan_domain(d->igloc_fluid, d->nel_fluid, d->nglob_fluid, patch_elems, growth, pre_f, pf);
    if (e.empty()) e = validate_plan(d->igloc_fluid, d->nel_fluid, d->nglob_fluid, pre_f, pf);
    if (!e.empty()) return fail(nullptr, AXG_ERR_BAD_DESC, "fluid plan: " + e);
  }
  info->n_patches_solid = ps.n_patches;
  info->n_patches_fluid = pf.n_patches;
  info->n_colours_solid = ps.n_colours;
  info->n_colours_fluid = pf.n_colours;
  info->max_subrounds_solid = ps.max_rounds;
  info->max_subrounds_fluid = pf.max_rounds;
  info->patch_points_solid = 0;
  for (const PatchMeta &m : ps.meta) info->patch_points_solid += m.n_pts;
  info->kernels_per_force = ps.n_colours;
  info->patch_elems_solid = ps.patch_elems;
  info->growth_solid = ps.growth;
  info->patch_elems_fluid = pf.patch_elems;
  info->growth_fluid = pf.growth;
  return AXG_OK;
}

int axg_time_stiffness(axg_handle *h, int32_t n, float *ms_avg) {
  if (!h || !ms_avg || n < 1) return fail(h, AXG_ERR_BAD_ARG, "bad argument");
  CK(cudaEventRecord(h->ev0, h->stream));
  for (int k = 0; k < n; ++k) enqueue_force(h, h->stream);
  CK(cudaEventRecord(h->ev1, h->stream));
  CK(cudaEventSynchronize(h->ev1));
  CK(cudaGetLastError());
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
  *ms_avg = ms / n;
  return AXG_OK;
}

void axg_destroy(axg_handle *h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  release(h);
  delete h;
}

int axg_device_check_report(int32_t *out8) {
  if (!out8) return fail(nullptr, AXG_ERR_BAD_ARG, "out8 is NULL");
#ifdef AXG_DEVICE_CHECKS
  cudaError_t e = cudaMemcpyFromSymbol(out8, g_axg_check, 8 * sizeof(int32_t));
  if (e != cudaSuccess) return fail(nullptr, AXG_ERR_CUDA, cudaGetErrorString(e));
  return AXG_OK;
#else
  std::memset(out8, 0, 8 * sizeof(int32_t));
  return fail(nullptr, AXG_ERR_UNSUPPORTED, "device checks are not compiled into this build");
#endif
}

const char *axg_last_error(axg_handle *h) { return h ? h->err.c_str() : g_create_error.c_str(); }

}  // extern "C"

namespace {
// One thread waits, through the kernels' own bounded wait, on an mbarrier that
// nothing arrives at and no copy targets; the wait must give up after about
// kWaitNs and record AXG_ERR_TIMEOUT.  No copy is in flight when it returns.
__global__ void wait_selftest_kernel(int32_t *err, unsigned long long *elapsed_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  fence_mbar_init();
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint64_t t0 = globaltimer_ns();
    const bool done = mbar_wait_bounded(&bar, 0u, err);
    *elapsed_ns = globaltimer_ns() - t0;
    if (done) atomicExch(err, -1);  // the phase cannot have completed
  }
}
}  // namespace

extern "C" int axg_selftest_wait_timeout(int32_t *status, double *elapsed_s) {
  if (!status || !elapsed_s) return fail(nullptr, AXG_ERR_BAD_ARG, "NULL argument");
  if (axg_device_count() < 1) return fail(nullptr, AXG_ERR_NO_DEVICE, "no CUDA device is visible");
  void *buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, 16);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMalloc");
  int32_t *err = static_cast<int32_t *>(buf);
  unsigned long long *ns = reinterpret_cast<unsigned long long *>(static_cast<char *>(buf) + 8);
  unsigned char host[16] = {};
  e = cudaMemset(buf, 0, 16);
  if (e == cudaSuccess) {
    wait_selftest_kernel<<<1, 32>>>(err, ns);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(host, buf, 16, cudaMemcpyDeviceToHost);
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "wait self-test");
  std::memcpy(status, host, 4);
  unsigned long long t = 0;
  std::memcpy(&t, host + 8, 8);
  *elapsed_s = 1e-9 * (double)t;
  return AXG_OK;
}

extern "C" {

int axg_set_wavefield_dump(axg_handle *h, const axg_dump_desc *dd) {
  if (!h || !dd) return fail(h, AXG_ERR_BAD_ARG, "NULL argument");
  if (h->pending) return fail(h, AXG_ERR_BAD_ARG, "the handle has queued steps");
  if (dd->dump_type < AXG_DUMP_NONE || dd->dump_type > AXG_DUMP_FULLFIELDS)
    return fail(h, AXG_ERR_BAD_ARG, "unknown dump_type");
  Dump &dp = h->dump;
  drop_graphs(h);
  if (dd->dump_type == AXG_DUMP_NONE) {
    dp.type = 0;
    return AXG_OK;
  }
  if (dd->strain_it < 1) return fail(h, AXG_ERR_BAD_ARG, "strain_it must be >= 1");
  if (dd->ibeg < 0 || dd->iend > 4 || dd->ibeg > dd->iend || dd->jbeg < 0 || dd->jend > 4 || dd->jbeg > dd->jend)
    return fail(h, AXG_ERR_BAD_ARG, "ibeg..iend, jbeg..jend must lie in 0..4");
  if (!dd->out || dd->capacity < 1) return fail(h, AXG_ERR_BAD_ARG, "no dump buffer");
  const float *sol[5] = {dd->DsDeta_over_J_sol, dd->DzDeta_over_J_sol, dd->DsDxi_over_J_sol, dd->DzDxi_over_J_sol,
                         dd->inv_s_solid};
  const float *flu[6] = {dd->DsDeta_over_J_flu, dd->DzDeta_over_J_flu, dd->DsDxi_over_J_flu, dd->DzDxi_over_J_flu,
                         dd->inv_s_fluid, dd->inv_rho_fluid};
  for (const float *a : sol)
    if (!a) return fail(h, AXG_ERR_BAD_ARG, "a solid data_pointwise array is NULL");
  if (h->nel_f > 0)
    for (const float *a : flu)
      if (!a) return fail(h, AXG_ERR_BAD_ARG, "a fluid data_pointwise array is NULL");
  int rc;
  const size_t es = 25 * (size_t)h->nel_s, ef = 25 * (size_t)std::max<int64_t>(h->nel_f, 0);
  if (!dp.gidx_s) {  // first use: numbering, axis flags, pointwise arrays on the device
    std::vector<int32_t> g(h->igloc_s.size());
    for (size_t p = 0; p < g.size(); ++p) g[p] = h->igloc_s[p] - 1;
    if ((rc = upload(h, &dp.gidx_s, g)) || (rc = upload(h, &dp.ax_s, h->axial_s))) return rc;
    for (int k = 0; k < 5; ++k)
      if ((rc = dalloc(h, &dp.pw_s[k], es))) return rc;
    if (h->nel_f > 0) {
      std::vector<int32_t> gf(h->igloc_f.size());
      for (size_t p = 0; p < gf.size(); ++p) gf[p] = h->igloc_f[p] - 1;
      if ((rc = upload(h, &dp.gidx_f, gf)) || (rc = upload(h, &dp.ax_f, h->axial_f))) return rc;
      for (int k = 0; k < 5; ++k)
        if ((rc = dalloc(h, &dp.pw_f[k], ef))) return rc;
      if ((rc = dalloc(h, &dp.inv_rho, ef))) return rc;
    }
    for (int k = 0; k < 2; ++k) {
      CK(cudaEventCreateWithFlags(&dp.ev_dump[k], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&dp.ev_copy[k], cudaEventDisableTiming));
    }
    if (!h->copy_stream) CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
  }
  for (int k = 0; k < 5; ++k)
    CK(cudaMemcpyAsync(dp.pw_s[k], sol[k], es * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  if (h->nel_f > 0) {
    for (int k = 0; k < 5; ++k)
      CK(cudaMemcpyAsync(dp.pw_f[k], flu[k], ef * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(dp.inv_rho, flu[5], ef * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  }
  const std::vector<std::string> fs = dump_fields(dd->dump_type, h->pole, false);
  const std::vector<std::string> ff = h->nel_f > 0 ? dump_fields(dd->dump_type, h->pole, true)
                                                    : std::vector<std::string>();
  dp.type = dd->dump_type;
  dp.strain_it = dd->strain_it;
  dp.src_mask = dd->src_dump_mask != 0;
  dp.ibeg = dd->ibeg;
  dp.iend = dd->iend;
  dp.jbeg = dd->jbeg;
  dp.jend = dd->jend;
  dp.ns = (int)fs.size();
  dp.nf = (int)ff.size();
  dp.np = (int64_t)(dd->iend - dd->ibeg + 1) * (dd->jend - dd->jbeg + 1);
  dp.floats = dp.np * ((int64_t)dp.ns * h->nel_s + (int64_t)dp.nf * std::max<int64_t>(h->nel_f, 0));
  dp.kwf = dd->kwf_mask != nullptr || dd->mapping_ijel_ikwf != nullptr;
  if (dp.kwf) {
    // the kernel wavefield point layout: the position each writing element
    // point has in its field, in the reference's element order
    if (!dd->kwf_mask || !dd->mapping_ijel_ikwf || dd->npoint_solid_kwf < 0 || dd->npoint_fluid_kwf < 0)
      return fail(h, AXG_ERR_BAD_ARG, "kwf_mask, mapping_ijel_ikwf and the kwf point counts go together");
    std::vector<int32_t> ps(es, -1), pf(ef, -1);
    for (size_t q = 0; q < es + ef; ++q) {
      if (!dd->kwf_mask[q]) continue;
      const bool fl = q >= es;
      const int64_t pos = (int64_t)dd->mapping_ijel_ikwf[q] - 1 - (fl ? dd->npoint_solid_kwf : 0);
      if (pos < 0 || pos >= (fl ? dd->npoint_fluid_kwf : dd->npoint_solid_kwf))
        return fail(h, AXG_ERR_BAD_ARG, "mapping_ijel_ikwf entry outside its domain's kwf points");
      (fl ? pf[q - es] : ps[q]) = (int32_t)pos;
    }
    if (!dp.kwf_s && (rc = dalloc(h, &dp.kwf_s, es))) return rc;
    CK(cudaMemcpyAsync(dp.kwf_s, ps.data(), es * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    if (ef > 0) {
      if (!dp.kwf_f && (rc = dalloc(h, &dp.kwf_f, ef))) return rc;
      CK(cudaMemcpyAsync(dp.kwf_f, pf.data(), ef * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    }
    dp.npt_s = dd->npoint_solid_kwf;
    dp.npt_f = ef > 0 ? dd->npoint_fluid_kwf : 0;
    dp.floats = (int64_t)dp.ns * dp.npt_s + (int64_t)dp.nf * dp.npt_f;
  }
  dp.out = dd->out;
  dp.capacity = dd->capacity;
  dp.names = fs;
  dp.names.insert(dp.names.end(), ff.begin(), ff.end());
  if (dp.floats > dp.slot_floats) {
    for (int k = 0; k < 2; ++k)
      if ((rc = dalloc(h, &dp.slot[k], (size_t)dp.floats))) return rc;
    dp.slot_floats = dp.floats;
  }
  CK(cudaStreamSynchronize(h->stream));
  return AXG_OK;
}

int axg_wavefield_dump_layout(axg_handle *h, int32_t *n_solid_fields, int32_t *n_fluid_fields,
                              int64_t *floats_per_snapshot, char *names, int32_t names_cap) {
  if (!h) return fail(nullptr, AXG_ERR_BAD_ARG, "handle is NULL");
  const Dump &dp = h->dump;
  if (n_solid_fields) *n_solid_fields = dp.type ? dp.ns : 0;
  if (n_fluid_fields) *n_fluid_fields = dp.type ? dp.nf : 0;
  if (floats_per_snapshot) *floats_per_snapshot = dp.type ? dp.floats : 0;
  if (names && names_cap > 0) {
    std::string all;
    if (dp.type)
      for (size_t k = 0; k < dp.names.size(); ++k) all += (k ? "," : "") + dp.names[k];
    const size_t n = std::min(all.size(), (size_t)names_cap - 1);
    std::memcpy(names, all.data(), n);
    names[n] = 0;
  }
  return AXG_OK;
}

}  // extern "C"

// ------------------------------------------------------------ batches

struct axg_batch {
  std::vector<axg_handle *> hs;
  int device = 0, num_sms = 1;
  SpecDev spec{};
  // resident CTAs of the batched solid kernels per (symplectic, pole, compensated, attenuated)
  int solid_ctas[2][3][2][2] = {};
  cudaStream_t stream = nullptr;
  // one step of every solve, captured with the plain Newmark solves' buffer
  // roles at parity 0 and at parity 1 (trade_buffers); steps alternate them
  cudaGraphExec_t graph[2] = {};
  cudaEvent_t ev_done = nullptr;
  bool pending = false;
  int64_t launches_per_step = 0;
  std::string err = "no error";
};

namespace {

int bfail(axg_batch *b, int code, const std::string &msg) {
  b->err = msg;
  return code;
}

#define BCK(call)                                                                                        \
  do {                                                                                                   \
    cudaError_t e_ = (call);                                                                             \
    if (e_ != cudaSuccess)                                                                               \
      return bfail(b, e_ == cudaErrorMemoryAllocation ? AXG_ERR_OOM : AXG_ERR_CUDA,                      \
                   fmt("%s: %s", #call, cudaGetErrorString(e_)));                                        \
  } while (0)

// Launches over the solves that `items` gives work (> 0 items), at most
// kMaxBatch solves per launch; returns the number of launches.
template <class W, class ItemsFn, class WorkFn, class LaunchFn>
int64_t for_batches(const std::vector<axg_handle *> &hs, ItemsFn items, WorkFn work, LaunchFn launch) {
  int64_t nl = 0;
  Many<W> m{};
  auto flush = [&]() {
    if (m.n > 0) {
      launch(m);
      ++nl;
    }
    m.n = 0;
    m.start[0] = 0;
  };
  for (axg_handle *h : hs) {
    const int32_t k = items(h);
    if (k <= 0) continue;
    m.w[m.n] = work(h);
    m.start[m.n + 1] = m.start[m.n] + k;
    if (++m.n == kMaxBatch) flush();
  }
  flush();
  return nl;
}

// A batched launch covers the solves taking part in one phase: the Newmark
// step (stage < 0) or stage `stage` of a symplectic step.
bool in_stage(const axg_handle *h, int stage) {
  return stage < 0 ? h->scheme == AXG_SCHEME_NEWMARK2 : h->scheme != AXG_SCHEME_NEWMARK2 && stage < h->nstages;
}
// the solve's solid and fluid state in that phase
void stage_states(axg_handle *h, int stage, StateArgs &ss, StateArgs &fs) {
  if (stage < 0) {
    ss = solid_state(h);
    fs = fluid_state(h);
  } else {
    symplectic_stage_states(h, stage, ss, fs);
  }
}

// the fluid's two passes for the solves of a phase, per class (non-monopole, compensated)
template <int NONMONO, bool KAHAN>
int64_t batch_fluid(axg_batch *b, int stage, cudaStream_t s) {
  auto mine = [&](axg_handle *h) {
    return in_stage(h, stage) && h->nel_f > 0 && (h->pole != AXG_MONOPOLE) == (NONMONO != 0) && h->kahan == KAHAN;
  };
  auto work = [&](axg_handle *h) {
    FluidArgs fa = fluid_args(h);
    if (stage >= 0) fa.fsmask = nullptr;  // symplectic_time_loop applies no free-surface mask
    StateArgs ss, fs;
    stage_states(h, stage, ss, fs);
    return FluidWork{fa, fs};
  };
  const int64_t ne = for_batches<FluidWork>(
      b->hs, [&](axg_handle *h) { return mine(h) ? (int32_t)h->nel_f : 0; }, work,
      [&](const Many<FluidWork> &m) {
        const unsigned g = fluid_elem_grid(m.start[m.n]);
        if (stage < 0)
          fluid_elem_kernel<NONMONO, MODE_NEWMARK, KAHAN, Many<FluidWork>><<<g, kFlElemThreads, 0, s>>>(m, b->spec);
        else
          fluid_elem_kernel<NONMONO, MODE_SYMPLECTIC, KAHAN, Many<FluidWork>><<<g, kFlElemThreads, 0, s>>>(m, b->spec);
      });
  const int64_t np = for_batches<FluidWork>(
      b->hs, [&](axg_handle *h) { return mine(h) ? (int32_t)h->nglob_f : 0; }, work,
      [&](const Many<FluidWork> &m) {
        const unsigned g = (unsigned)((m.start[m.n] + 255) / 256);
        if (stage < 0) fluid_point_kernel<NONMONO, MODE_NEWMARK, KAHAN, Many<FluidWork>><<<g, 256, 0, s>>>(m);
        else fluid_point_kernel<NONMONO, MODE_SYMPLECTIC, KAHAN, Many<FluidWork>><<<g, 256, 0, s>>>(m);
      });
  return ne + np;
}

// a solve's colour work with its attenuation data (attenuated batches)
struct AnelPatchWork {
  PatchWork pw;
  AnelArgs an;
};

template <int POLE, int MODE, bool KAHAN, bool ANEL>
int64_t batch_solid_colour(axg_batch *b, int stage, int c, cudaStream_t s) {
  const int pole = POLE == POLE_MONO ? AXG_MONOPOLE : POLE == POLE_DI ? AXG_DIPOLE : AXG_QUADPOLE;
  return for_batches<AnelPatchWork>(
      b->hs,
      [&](axg_handle *h) {
        const bool mine = in_stage(h, stage) && c < h->ps.n_colours && h->pole == pole && h->kahan == KAHAN &&
                          h->anel == ANEL;
        return mine ? h->ps.colour_start[c + 1] - h->ps.colour_start[c] : 0;
      },
      [&](axg_handle *h) {
        DomainArgs a = domain_args(h->ds, h->ps);
        a.patch_begin = h->ps.colour_start[c];
        StateArgs ss, fs;
        stage_states(h, stage, ss, fs);
        return AnelPatchWork{PatchWork{a, ss}, h->an};
      },
      [&](const Many<AnelPatchWork> &mw) {
        Many<PatchWork> m{};
        m.n = mw.n;
        std::memcpy(m.start, mw.start, sizeof(m.start));
        for (int q = 0; q < mw.n; ++q) m.w[q] = mw.w[q].pw;
        const int grid = std::min(m.start[m.n], b->solid_ctas[MODE == MODE_SYMPLECTIC][POLE][KAHAN][ANEL]);
        constexpr int smem = solid_smem_bytes<POLE, MODE, ANEL, KAHAN>();
        if constexpr (ANEL) {
          AnelBatch an{};
          for (int q = 0; q < mw.n; ++q) an.a[q] = mw.w[q].an;
          solid_anel_batch_kernel<POLE, MODE, KAHAN><<<grid, kThreads, smem, s>>>(m, b->spec, an);
        } else {
          solid_batch_kernel<POLE, MODE, KAHAN><<<grid, kThreads, smem, s>>>(m, b->spec);
        }
      });
}

// colour c of the solid, every pole and precision mode, plain and attenuated
template <int MODE>
int64_t batch_solid_colours(axg_batch *b, int stage, int c, cudaStream_t s) {
  return batch_solid_colour<POLE_MONO, MODE, false, false>(b, stage, c, s) +
         batch_solid_colour<POLE_MONO, MODE, true, false>(b, stage, c, s) +
         batch_solid_colour<POLE_DI, MODE, false, false>(b, stage, c, s) +
         batch_solid_colour<POLE_DI, MODE, true, false>(b, stage, c, s) +
         batch_solid_colour<POLE_QUAD, MODE, false, false>(b, stage, c, s) +
         batch_solid_colour<POLE_QUAD, MODE, true, false>(b, stage, c, s) +
         batch_solid_colour<POLE_MONO, MODE, false, true>(b, stage, c, s) +
         batch_solid_colour<POLE_MONO, MODE, true, true>(b, stage, c, s) +
         batch_solid_colour<POLE_DI, MODE, false, true>(b, stage, c, s) +
         batch_solid_colour<POLE_DI, MODE, true, true>(b, stage, c, s) +
         batch_solid_colour<POLE_QUAD, MODE, false, true>(b, stage, c, s) +
         batch_solid_colour<POLE_QUAD, MODE, true, true>(b, stage, c, s);
}

template <int POLE>
int64_t batch_to_solid(axg_batch *b, int stage, cudaStream_t s) {
  const int pole = POLE == POLE_MONO ? AXG_MONOPOLE : POLE == POLE_DI ? AXG_DIPOLE : AXG_QUADPOLE;
  return for_batches<ToSolidWork>(
      b->hs,
      [&](axg_handle *h) { return in_stage(h, stage) && h->nel_f > 0 && h->pole == pole ? h->to_solid.n : 0; },
      [&](axg_handle *h) {
        StateArgs ss, fs;
        stage_states(h, stage, ss, fs);
        return ToSolidWork{h->to_solid, fs, ss};
      },
      [&](const Many<ToSolidWork> &m) {
        couple_to_solid_kernel<POLE, Many<ToSolidWork>><<<(m.start[m.n] + 255) / 256, 256, 0, s>>>(m);
      });
}

template <int DIPOLE>
int64_t batch_to_fluid(axg_batch *b, int stage, cudaStream_t s) {
  return for_batches<ToFluidWork>(
      b->hs,
      [&](axg_handle *h) {
        return in_stage(h, stage) && h->nel_f > 0 && (h->pole == AXG_DIPOLE) == (DIPOLE != 0) ? h->to_fluid.n : 0;
      },
      [&](axg_handle *h) {
        StateArgs ss, fs;
        stage_states(h, stage, ss, fs);
        return ToFluidWork{h->to_fluid, ss, h->ff, h->ds.axmask};
      },
      [&](const Many<ToFluidWork> &m) {
        couple_to_fluid_kernel<DIPOLE, Many<ToFluidWork>><<<(m.start[m.n] + 255) / 256, 256, 0, s>>>(m);
      });
}

// One phase of the solves taking part in it, in the order of enqueue_step
// (enqueue_step_symplectic for a stage): coupling into the fluid, fluid
// colours, coupling into the solid, solid colours.
template <int MODE>
int64_t enqueue_batch_phase(axg_batch *b, int stage, cudaStream_t s) {
  int64_t nl = batch_to_fluid<0>(b, stage, s) + batch_to_fluid<1>(b, stage, s);
  int sc = 0;
  for (axg_handle *h : b->hs)
    if (in_stage(h, stage)) sc = std::max(sc, h->ps.n_colours);
  nl += batch_fluid<0, false>(b, stage, s) + batch_fluid<0, true>(b, stage, s) + batch_fluid<1, false>(b, stage, s) +
        batch_fluid<1, true>(b, stage, s);
  nl += batch_to_solid<POLE_MONO>(b, stage, s) + batch_to_solid<POLE_DI>(b, stage, s) +
        batch_to_solid<POLE_QUAD>(b, stage, s);
  for (int c = 0; c < sc; ++c) nl += batch_solid_colours<MODE>(b, stage, c, s);
  return nl;
}

// One step of every solve: the Newmark solves' step, the symplectic solves'
// stages (stage i of every solve with more than i stages in one phase), their
// final drifts and memory variables, then the seismograms and step counters.
int64_t enqueue_batch_step(axg_batch *b, cudaStream_t s) {
  int64_t nl = enqueue_batch_phase<MODE_NEWMARK>(b, -1, s);
  for (axg_handle *h : b->hs) trade_buffers(h);  // the plain Newmark solves' state after the step
  int ns = 0;
  for (axg_handle *h : b->hs) ns = std::max(ns, h->scheme != AXG_SCHEME_NEWMARK2 ? h->nstages : 0);
  for (int i = 0; i < ns; ++i) nl += enqueue_batch_phase<MODE_SYMPLECTIC>(b, i, s);
  if (ns > 0) {
    nl += for_batches<DriftWork>(
        b->hs, [](axg_handle *h) { return h->scheme != AXG_SCHEME_NEWMARK2 ? drift_points(h) : 0; },
        [](axg_handle *h) { return drift_work(h); },
        [&](const Many<DriftWork> &m) { drift_kernel<Many<DriftWork>><<<(m.start[m.n] + 255) / 256, 256, 0, s>>>(m); });
    for (axg_handle *h : b->hs)
      if (h->scheme != AXG_SCHEME_NEWMARK2 && h->anel) {
        launch_anel_memvar_pole(h, s);
        ++nl;
      }
  }
  nl += for_batches<RecWork>(
      b->hs, [](axg_handle *) { return 1; }, [](axg_handle *h) { return rec_work(h, solid_state(h)); },
      [&](const Many<RecWork> &m) { receivers_kernel<Many<RecWork>><<<m.n, 256, 0, s>>>(m); });
  return nl;
}

// kernel parameters are limited to 32764 bytes
static_assert(sizeof(Many<PatchWork>) + sizeof(SpecDev) + sizeof(AnelBatch) <= 32000 &&
                  sizeof(Many<FluidWork>) + sizeof(SpecDev) <= 32000 &&
                  sizeof(Many<ToSolidWork>) <= 32000 && sizeof(Many<DriftWork>) <= 32000 &&
                  sizeof(Many<ToFluidWork>) <= 32000 && sizeof(Many<RecWork>) <= 32000,
              "a batched launch's descriptors must fit the kernel parameter space");

// the step counters of up to kMaxBatch solves
struct IterSet {
  int32_t n;
  int32_t *ctr[kMaxBatch];
  int32_t first[kMaxBatch];
};
__global__ void set_iters_kernel(const __grid_constant__ IterSet a) {
  if ((int)threadIdx.x < a.n) *a.ctr[threadIdx.x] = a.first[threadIdx.x];
}

template <int POLE, int MODE, bool KAHAN, bool ANEL>
int prepare_batch_kernel(axg_batch *b, axg_handle *h) {
  int *ctas = &b->solid_ctas[MODE == MODE_SYMPLECTIC][POLE][KAHAN][ANEL];
  constexpr int smem = solid_smem_bytes<POLE, MODE, ANEL, KAHAN>();
  int rc;
  if constexpr (ANEL) rc = prepare_kernel_fn(h, solid_anel_batch_kernel<POLE, MODE, KAHAN>, smem, ctas);
  else rc = prepare_kernel_fn(h, solid_batch_kernel<POLE, MODE, KAHAN>, smem, ctas);
  if (rc) b->err = h->err;
  return rc;
}

template <int POLE, int MODE>
int prepare_batch_kernels(axg_batch *b, axg_handle *h) {
  if (h->anel)
    return h->kahan ? prepare_batch_kernel<POLE, MODE, true, true>(b, h) : prepare_batch_kernel<POLE, MODE, false, true>(b, h);
  return h->kahan ? prepare_batch_kernel<POLE, MODE, true, false>(b, h) : prepare_batch_kernel<POLE, MODE, false, false>(b, h);
}

// the batched solid kernel a solve of the batch launches
template <int MODE>
int prepare_batch_mode(axg_batch *b, axg_handle *h) {
  if (h->pole == AXG_MONOPOLE) return prepare_batch_kernels<POLE_MONO, MODE>(b, h);
  if (h->pole == AXG_DIPOLE) return prepare_batch_kernels<POLE_DI, MODE>(b, h);
  return prepare_batch_kernels<POLE_QUAD, MODE>(b, h);
}

int batch_create_impl(axg_batch *b, axg_handle *const *hs, int32_t n) {
  if (!hs || n < 1) return bfail(b, AXG_ERR_BAD_ARG, "axg_batch_create: no handles");
  for (int k = 0; k < n; ++k) {
    axg_handle *h = hs[k];
    if (!h) return bfail(b, AXG_ERR_BAD_ARG, fmt("axg_batch_create: handle %d is NULL", k));
    for (int q = 0; q < k; ++q)
      if (hs[q] == h) return bfail(b, AXG_ERR_BAD_ARG, fmt("axg_batch_create: handle %d appears twice", k));
    if (k > 0 && (h->device != hs[0]->device || std::memcmp(&h->spec, &hs[0]->spec, sizeof(SpecDev)) != 0))
      return bfail(b, AXG_ERR_BAD_ARG,
                   fmt("axg_batch_create: solve %d is on another device or has other GLL matrices", k));
    if (h->pending) return bfail(b, AXG_ERR_BAD_ARG, fmt("axg_batch_create: solve %d has queued steps", k));
    if (h->dump.type)
      return bfail(b, AXG_ERR_UNSUPPORTED, fmt("axg_batch_create: solve %d dumps wavefields (it runs alone)", k));
    if (h->ckpt.check_it > 0)
      return bfail(b, AXG_ERR_UNSUPPORTED,
                   fmt("axg_batch_create: solve %d checkpoints its seismograms (it runs alone)", k));
    if (h->anel_full)
      return bfail(b, AXG_ERR_UNSUPPORTED,
                   fmt("axg_batch_create: solve %d has attenuation at every GLL point (it runs alone)", k));
    b->hs.push_back(h);
  }
  b->device = hs[0]->device;
  b->spec = hs[0]->spec;
  b->num_sms = hs[0]->num_sms;
  for (axg_handle *h : b->hs) {
    const int rc = h->scheme == AXG_SCHEME_NEWMARK2 ? prepare_batch_mode<MODE_NEWMARK>(b, h)
                                                    : prepare_batch_mode<MODE_SYMPLECTIC>(b, h);
    if (rc) return rc;
  }
  BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  BCK(cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming));
  // the solves' buffers in their parity-0 roles (each solve's stream is idle)
  for (axg_handle *h : b->hs) {
    BCK(normalize_buffers(h, h->stream));
    BCK(cudaStreamSynchronize(h->stream));
  }
  // one step, captured once per parity; every step of every run replays one
  for (int p = 0; p < 2; ++p) {
    cudaGraph_t g;
    BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    b->launches_per_step = enqueue_batch_step(b, b->stream);  // (trades the buffers: parity p + 1)
    const cudaError_t le = cudaGetLastError();
    const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (le != cudaSuccess || ce != cudaSuccess) {
      if (ce == cudaSuccess) cudaGraphDestroy(g);
      if (p == 0)
        for (axg_handle *h : b->hs) trade_buffers(h);  // back to parity 0
      return bfail(b, AXG_ERR_CUDA, fmt("batch step capture: %s", cudaGetErrorString(le != cudaSuccess ? le : ce)));
    }
    const cudaError_t ie = cudaGraphInstantiate(&b->graph[p], g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess && p == 0)
      for (axg_handle *h : b->hs) trade_buffers(h);
    BCK(ie);
  }
  return AXG_OK;
}

void batch_release(axg_batch *b) {
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (cudaGraphExec_t g : b->graph)
    if (g) cudaGraphExecDestroy(g);
  if (b->ev_done) cudaEventDestroy(b->ev_done);
  if (b->stream) cudaStreamDestroy(b->stream);
}

// the solves' flags once the batch's work completed; the first error found
int batch_flags(axg_batch *b) {
  for (size_t k = 0; k < b->hs.size(); ++k) {
    const int rc = check_flags(b->hs[k]);
    if (rc) return bfail(b, rc, fmt("solve %d: %s", (int)k, b->hs[k]->err.c_str()));
  }
  return AXG_OK;
}

}  // namespace

extern "C" {

int axg_batch_create(axg_handle *const *hs, int32_t n, axg_batch **out) {
  if (!out) return fail(nullptr, AXG_ERR_BAD_ARG, "out is NULL");
  *out = nullptr;
  axg_batch *b = new axg_batch();
  const int rc = batch_create_impl(b, hs, n);
  if (rc) {
    g_create_error = b->err;
    batch_release(b);
    delete b;
    return rc;
  }
  *out = b;
  return AXG_OK;
}

int axg_batch_run_async(axg_batch *b, const int32_t *first_iters, int32_t n_iter) {
  if (!b || !first_iters) return b ? bfail(b, AXG_ERR_BAD_ARG, "first_iters is NULL") : AXG_ERR_BAD_ARG;
  if (b->pending) return bfail(b, AXG_ERR_BAD_ARG, "the batch has queued steps (axg_batch_poll / axg_batch_wait)");
  if (n_iter < 0) return bfail(b, AXG_ERR_BAD_ARG, "n_iter < 0");
  const int n = (int)b->hs.size();
  for (int k = 0; k < n; ++k) {
    const axg_handle *h = b->hs[k];
    if (first_iters[k] < 1 || (int64_t)first_iters[k] + n_iter - 1 > h->niter)
      return bfail(b, AXG_ERR_BAD_ARG, fmt("solve %d: iterations %d..%d outside 1..niter=%d", k, first_iters[k],
                                           first_iters[k] + n_iter - 1, h->niter));
  }
  if (n_iter == 0) return AXG_OK;
  // the batch follows the work already queued on each solve's stream
  for (axg_handle *h : b->hs) {
    BCK(cudaEventRecord(h->ev_done, h->stream));
    BCK(cudaStreamWaitEvent(b->stream, h->ev_done, 0));
    BCK(normalize_buffers(h, b->stream));  // the graphs' parity 0
    BCK(refresh_predicted(h, b->stream));
  }
  for (int k0 = 0; k0 < n; k0 += kMaxBatch) {
    IterSet a{};
    a.n = std::min(kMaxBatch, n - k0);
    for (int q = 0; q < a.n; ++q) {
      a.ctr[q] = b->hs[k0 + q]->iter;
      a.first[q] = first_iters[k0 + q];
    }
    set_iters_kernel<<<1, kMaxBatch, 0, b->stream>>>(a);
  }
  BCK(cudaGetLastError());
  for (int32_t q = 0; q < n_iter; ++q) {
    BCK(cudaGraphLaunch(b->graph[q & 1], b->stream));
    for (axg_handle *h : b->hs) trade_buffers(h);
  }
  BCK(cudaEventRecord(b->ev_done, b->stream));
  // and each solve's later work follows the batch
  for (axg_handle *h : b->hs) BCK(cudaStreamWaitEvent(h->stream, b->ev_done, 0));
  b->pending = true;
  return AXG_OK;
}

int axg_batch_poll(axg_batch *b, int32_t *done) {
  if (!b || !done) return b ? bfail(b, AXG_ERR_BAD_ARG, "done is NULL") : AXG_ERR_BAD_ARG;
  *done = 1;
  if (!b->pending) return AXG_OK;
  const cudaError_t e = cudaEventQuery(b->ev_done);
  if (e == cudaErrorNotReady) {
    *done = 0;
    return AXG_OK;
  }
  b->pending = false;
  BCK(e);
  return batch_flags(b);
}

int axg_batch_wait(axg_batch *b) {
  if (!b) return AXG_ERR_BAD_ARG;
  const bool was = b->pending;
  b->pending = false;
  BCK(cudaStreamSynchronize(b->stream));
  return was ? batch_flags(b) : AXG_OK;
}

int axg_batch_launches_per_step(axg_batch *b, int64_t *n) {
  if (!b || !n) return b ? bfail(b, AXG_ERR_BAD_ARG, "n is NULL") : AXG_ERR_BAD_ARG;
  *n = b->launches_per_step;
  return AXG_OK;
}

void axg_batch_destroy(axg_batch *b) {
  if (!b) return;
  batch_release(b);
  delete b;
}

const char *axg_batch_last_error(axg_batch *b) { return b ? b->err.c_str() : g_create_error.c_str(); }

}  // extern "C"

