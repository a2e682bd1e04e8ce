// axg_plan.h -- host-side planning of the patch-coloured assembly.
//
// The reference assembles element contributions with a sequential
// gather/scatter over igloc (SOLVER/commun.F90:99-158).  On the GPU every
// CTA owns a *patch* of elements: it gathers the patch's global points into
// shared memory once, accumulates its elements' contributions there in a
// fixed order (elements are split into sub-rounds that share no point), and
// writes the patch sums back.  Patches that share a point get different
// colours and run in different launches, so the global write-back is
// race-free without atomics, and the order in which a point's partial sums
// are added (pre-pass, then colour 0, 1, ...) is fixed: results are
// bit-reproducible run to run.
//
// The planner is plain C++ with no CUDA dependency so that it can be checked
// on a machine without a GPU.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace axg {

constexpr int kMaxPatchElems = 64;      // elements per patch (upper bound)
constexpr int kMaxSubrounds = 12;       // conflict-free element groups per patch
// points per patch: sized so that three Newmark CTAs fit on an SM (an 8 x 8
// patch of a structured grid has 33^2 = 1089 points); growth stops at it.
// A multiple of 4 (the point words of a patch are copied in 16-byte units).
constexpr int kMaxPatchPoints = 1092;
constexpr int64_t kTunePrefix = 65536;  // elements the patch-size tuner plans

enum PatchGrowth { kGrowCompact = 0, kGrowLayered = 1 };

// bits of a patch point word: global index in the low 28 bits
constexpr uint32_t kPtIndexMask = 0x0FFFFFFFu;
constexpr uint32_t kPtFirst = 1u << 28;   // first writer: store, do not read partial sum
constexpr uint32_t kPtLast = 1u << 29;    // last writer: the sum is final
constexpr uint32_t kPtSource = 1u << 30;  // point carries a solid source term
constexpr uint32_t kPtAxis = 1u << 31;    // point on the axis (ipol = 0 of an axial element); set by the host
constexpr uint32_t kPtPad = 0xFFFFFFFFu;  // padding after a patch's words (each patch starts 16-byte aligned)

struct PatchMeta {            // 32 bytes, device layout
  int32_t elem_start;         // first element (launch order)
  int32_t pt_start;           // first point word
  uint16_t n_elems;
  uint16_t n_pts;
  uint8_t n_rounds;
  uint8_t round_end[19];      // cumulative element counts per sub-round (<= kMaxSubrounds used)
};
static_assert(sizeof(PatchMeta) == 32, "PatchMeta must be 32 bytes");

struct DomainPlan {
  int64_t nel = 0, nglob = 0;
  int patch_elems = 0;
  int growth = kGrowCompact;
  int32_t n_patches = 0;
  int32_t n_colours = 0;
  int32_t max_rounds = 0;
  int32_t max_pts = 0;
  std::vector<int32_t> patch_of_elem;    // nel (reference element order)
  std::vector<int32_t> colour_of_patch;  // n_patches (creation order)
  std::vector<int32_t> colour_start;     // n_colours+1 offsets into launch order of patches
  std::vector<PatchMeta> meta;           // n_patches, launch order
  std::vector<int32_t> elem_order;       // nel: reference element (0-based) at each launch slot
  std::vector<uint32_t> pt_words;        // patch point words, each patch padded to a multiple of 4
  // internal point numbering: the point words and every per-point device
  // array use new_of_old[g] for the reference's (0-based) point g
  std::vector<int32_t> new_of_old, old_of_new;
  std::vector<uint16_t> elem_pts;        // 25*nel, launch order: patch-local point index
  int64_t total_pts = 0;
};

// Builds patches of up to patch_elems elements (growth: kGrowCompact or
// kGrowLayered over the point-sharing element graph), merges fragments,
// colours the patches, splits each patch into sub-rounds and fills the point
// words.
//   igloc     : 25*nel 1-based global indices (walk ipol fastest)
//   prepass   : per global point, 1 if a pre-pass kernel writes it first
//               (solid-fluid coupling), may be empty
// Returns an empty string on success, else the reason.
// renumber: give points an internal numbering in which the points held by
// the same patches are contiguous (else the identity).
std::string build_plan(const int32_t *igloc, int64_t nel, int64_t nglob, int patch_elems, int growth,
                       const std::vector<uint8_t> &prepass, DomainPlan &plan, bool renumber = true);

// Model cost of a plan in 1/256 warp iterations of the patch kernels.
int64_t plan_cost(const DomainPlan &plan);

// Model time of a plan's colour launches when they do not fill the GPU:
// per colour, the largest sum over one CTA's patches (patch i of a colour
// goes to CTA i mod ctas) of (elements + overhead), summed over the colours,
// in element iterations.  overhead: a patch's fixed cost (gather, write-back,
// barriers) in element iterations, about 40 for the elastic kernels and 20
// for the attenuated one, whose elements cost twice as much (fitted to step
// times of the PREM meshes at 50, 25 and 10 s over patch sizes 8 to 64).
constexpr int kPatchOverheadElastic = 40, kPatchOverheadAnelastic = 20;
int64_t plan_latency(const DomainPlan &plan, int ctas, int overhead);

// Patch-size tuner: picks (patch_elems, growth).  With ctas = 0, or a mesh
// of at least kTuneFullRounds rounds of 64-element patches per colour over
// `ctas` resident CTAs, by least plan_cost on the first kTunePrefix
// elements: the launches are full and bandwidth-bound.  Below that, by least
// plan_latency of the whole mesh over sizes down to 8 elements: a colour is
// about one round of patches, and smaller patches spread it over more CTAs.
// patch_elems > 0 or growth >= 0 fix that choice.
constexpr int kTuneFullRounds = 2;
std::string tune_plan(const int32_t *igloc, int64_t nel, int64_t nglob, int patch_elems, int growth,
                      int *best_pe, int *best_growth, int ctas = 0, int overhead = kPatchOverheadElastic);

// Checks the invariants the kernels rely on (used by the tests and by
// axg_create in debug builds): every element in exactly one patch, no two
// patches of one colour share a point, no two elements of one sub-round share
// a point, first/last flags consistent.  Returns "" when valid.
std::string validate_plan(const int32_t *igloc, int64_t nel, int64_t nglob,
                          const std::vector<uint8_t> &prepass, const DomainPlan &plan);

}  // namespace axg
