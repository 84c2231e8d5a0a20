// extern "C" entry points of libsph_gb300 (declared in include/sph_gb300.h).
//
// The handle owns every device buffer (allocated once in sph_create); the
// per-step work is stream-ordered and allocation-free, so a sequence of steps
// is captured once into a CUDA graph and replayed.
#include <climits>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "sph_internal.cuh"

using namespace sph;

namespace {
thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return 0;
  return fail((int)SPH_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace

struct SphHandle {
  SphConfig cfg{};
  int n_cases = 0;
  std::vector<SphCase> cases;
  std::vector<CaseDev> hc;
  CaseDev* dc = nullptr;
  long long* case_off_d = nullptr;
  long long N = 0, C = 0;
  // buf[0] holds the state in the order of the last binning; buf[1] is the
  // scratch copy a rebuild sorts from, so buffer addresses never change and
  // one captured step serves every step
  Buffers buf[2]{};
  float4* R4 = nullptr;
  float4* UT4 = nullptr;
  float4* R4e = nullptr;   // evolved density before renormalisation
  WallLayer layer{};         // wall normals recomputed each step (layer.n > 0)
  float4* layer_pts = nullptr;
  int* layer_start = nullptr;
  float4* dscr = nullptr;  // delta-SPH density scratch (5 planes of N)
  int* cellid = nullptr;
  int *count = nullptr, *start = nullptr, *keyc = nullptr, *keys = nullptr;
  int *tsrc = nullptr, *tkey = nullptr, *tcell = nullptr, *scan_tmp = nullptr;
  int* rowcnt = nullptr;
  long long* rowoff = nullptr;  // 64-bit edge offsets per sender
  int *nbr = nullptr, *nbr_cnt = nullptr;
  int kmax = kListSlots;  // neighbour-list slots per particle
  int *vl = nullptr, *vcnt = nullptr;  // Verlet candidates
  int kv = kVerletMinSlots;          // Verlet slots per particle
  float4* rref = nullptr;              // positions at the last rebuild
  int* cref_count = nullptr;           // per-step occupancy of the reference's cells
  long long ref_cells = 0;
  unsigned* vflag = nullptr;           // [0] a rebuild is due, [1] sph_advance: positions changed
  unsigned long long* rebuilds_d = nullptr;  // rebuilds run inside graph replays
  long long rebuilds_h = 0;                  // rebuilds run eagerly
  int rebuild_launches = 0;                  // kernels of one rebuild
  unsigned char* stage = nullptr;  // device copies of pinned host fields (sph_advance)
  size_t stage_slot = 0;
  // the staging copies are spread over a few streams (several copy engines)
  static constexpr int kCopyStreams = 4;
  cudaStream_t cs[kCopyStreams] = {};
  cudaEvent_t fork = nullptr, join[kCopyStreams] = {};
  int block = 256;        // threads per block of the forward passes
  int force_variant = SPH_FORCE_GATHER;  // lean force pass: gathered or staged senders
  int lean = 0;           // served by the lean passes (sph_lean.cu): list format
  unsigned* status = nullptr;
  unsigned long long* edgecnt = nullptr;
  int* case_max = nullptr;  // allocate: largest reference-cell occupancy per case
  int* inv = nullptr;       // sorted position of each original index (valid once binned)
  const float* g_arr = nullptr;
  // binned: a binning (order, cells, inverse permutation) exists; lists: the
  // candidate lists fit the current positions; fresh: the binning itself is
  // of the current positions (no step since)
  bool has_state = false, binned = false, lists = false, fresh = false, from_forward = false,
       pending_bc = false;
  cudaStream_t hs = nullptr, hs2 = nullptr;  // capture streams (step, rebuild body)
  cudaGraphExec_t gexec = nullptr;           // one steady step
  const float* graph_g_arr = nullptr;
  cudaGraphExec_t gadv = nullptr;            // sph_advance: kick, decide, rebuild
  const float* gadv_g_arr = nullptr;
  int launch_count = 0;       // kernel launches of the last step
  cudaEvent_t* ev = nullptr;  // phase events while profiling
  // adjoint tape: per recorded step the sorted order, P4, U4, R4 and the
  // neighbour list of its forward pass
  int tape_slots = 0;
  int *t_orig = nullptr, *t_meta = nullptr;
  float4 *t_P4 = nullptr, *t_U4 = nullptr, *t_V4 = nullptr, *t_R4 = nullptr;
  int *t_nbr = nullptr, *t_cnt = nullptr;
  float4* t_scr = nullptr;              // reverse scratch: 8 planes of N
  float *t_la = nullptr, *t_lb = nullptr;  // the step inputs' dudt/dvdt adjoints
  // device snapshots of the state a steady handle carries between steps
  int snap_slots = 0;
  unsigned char* snap = nullptr;
  size_t snap_stride = 0;
  std::vector<char> snap_ok;
  std::vector<int> snap_fmt;  // list format of the passes when the slot was saved
  std::vector<void*> allocs;

  template <typename T>
  int alloc(T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) return cuda_check(e, "cudaMalloc");
    allocs.push_back(q);
    *p = (T*)q;
    return 0;
  }

  LaunchCtx ctx(cudaStream_t st) const {
    LaunchCtx L;
    L.stream = st;
    L.dim = cfg.dim;
    L.kernel = cfg.kernel;
    L.solver = cfg.solver;
    L.rho_evol = cfg.is_rho_evol;
    L.bc_trick = cfg.is_bc_trick;
    L.free_slip = cfg.is_free_slip;
    L.mask_self = cfg.mask_self;
    L.kahan = cfg.kahan;
    L.N = N;
    L.n_cases = n_cases;
    L.cases = dc;
    L.status = status;
    L.nbr = nbr;
    L.nbr_cnt = nbr_cnt;
    L.kmax = kmax;
    L.vl = vl;
    L.vcnt = vcnt;
    L.kv = kv;
    L.rref = rref;
    L.cref_count = cref_count;
    L.vflag = vflag;
    L.canonical = cfg.canonical_order;
    L.inv = inv;
    L.rho_renorm = cfg.is_rho_renorm;
    L.heat = cfg.is_heat_conduction;
    L.layer = layer;
    L.R4e = R4e;
    L.dscr = dscr;
    L.block = block;
    L.lean = lean;
    L.force_variant = force_variant;
    L.c1 = hc[0];
    L.launches = const_cast<int*>(&launch_count);
    L.ev = ev;
    return L;
  }
};

void sph::set_last_error(const std::string& msg) { g_last_error = msg; }

int sph::host_error() noexcept {
  try {
    try {
      throw;
    } catch (const std::bad_alloc&) {
      g_last_error = "host memory exhausted";
    } catch (const std::exception& e) {
      g_last_error = std::string("host error: ") + e.what();
    } catch (...) {
      g_last_error = "host error";
    }
  } catch (...) {
    // recording the message itself failed; the status bit still reports it
  }
  return (int)SPH_ERR_HOST;
}

// Per-case float32 constants, rounded the way the reference's float32
// program rounds its Python-float parameters (weak types become float32).
int sph::make_case(const SphConfig& cfg, const SphCase& in, long long p_off, long long cell_off,
              CaseDev& c, std::string& err, bool fine_cells) {
  std::memset(&c, 0, sizeof(c));
  const int dim = cfg.dim;
  const float cut = (float)in.r_cutoff + 0.0f;
  if (!(cut > 0.0f)) {
    err = "r_cutoff must be positive";
    return -1;
  }
  bool use_cells = true;
  int nc[3] = {1, 1, 1};
  for (int d = 0; d < 3; ++d) {
    const float box = d < dim ? (float)in.box[d] : 1.0f;
    c.box[d] = box;
    c.half[d] = box * 0.5f;
    if (d >= dim) continue;
    if (!(box > 0.0f)) {
      err = "box sides must be positive";
      return -1;
    }
    // _cell_dimensions (jax_md/partition.py:128-130) and the cell-list test (:935)
    if (!(cut < box / 3.0f)) use_cells = false;
    const float cps = std::floor(box / cut);
    nc[d] = cps >= 3.0f ? (int)cps : 1;
    c.cell_size[d] = nc[d] > 1 ? box / cps : box;
  }
  c.use_cells = use_cells;
  // Fast membership test. The minimum-image difference of two positions in
  // [0, L] differs from the reference's float32 periodic displacement by at
  // most ~3.3 ulp(L) per component, so their squared norms near the cutoff
  // differ by at most ~20 ulp(L) * cutoff plus a few roundings of cutoff^2.
  // Inside the band cut_sq * (1 +- rel) the reference metric decides.
  bool fast = true;
  float lmax = 0.f;
  for (int d = 0; d < dim; ++d) {
    fast = fast && nc[d] >= 5;
    lmax = c.box[d] > lmax ? c.box[d] : lmax;
    c.inv_box[d] = 1.0f / c.box[d];
  }
  const double rel = std::ldexp(24.0 * lmax / cut + 8.0, -23);
  c.fast = fast && rel < 0.25;
  c.cutoff_sq = cut * cut;
  if (c.fast) {
    c.cut_lo = (float)(c.cutoff_sq * (1.0 - rel));
    c.cut_hi = (float)(c.cutoff_sq * (1.0 + rel));
    // rows are trimmed to a sphere a little larger than the band's outer edge
    c.trim_r2 = (float)(c.cutoff_sq * (1.0 + rel) * (1.0 + std::ldexp(1.0, -20)));
    c.trim_m = (float)std::ldexp((double)lmax, -17);
  } else {  // every candidate takes the reference metric
    c.cut_lo = -1.0f;
    c.cut_hi = INFINITY;
  }
  // Fast cases are binned into half-size cells (fewer candidates per
  // receiver: the walk covers trimmed rows of half cells instead of +-1
  // reference cell). It reaches 3 half cells on each side: the reference's
  // candidates of a receiver in the lower half of its cell extend 3 half
  // cells up, and where the reference cell is the cutoff to within rounding a
  // sender at the cutoff distance can lie there.
  long long ncell = 1;
  for (int d = 0; d < 3; ++d) {
    const int sub = (fine_cells && c.fast && nc[d] > 1) ? 2 : 1;
    c.sub[d] = sub;
    c.nc[d] = nc[d] * sub;
    c.rad[d] = nc[d] > 1 ? (sub == 2 ? 3 : 1) : 0;
    if (sub == 2) c.cell_size[d] = c.cell_size[d] * 0.5f;
    c.inv_cs[d] = 1.0f / c.cell_size[d];
    c.mult[d] = (int)ncell;
    ncell *= c.nc[d];
  }
  if (ncell > INT_MAX / 2) {
    err = "too many cells";
    return -1;
  }
  c.ncell = (int)ncell;
  c.ncref = (int)(ncell / ((long long)c.sub[0] * c.sub[1] * c.sub[2]));
  // Verlet candidate list. Without a skin (or without the fast test) the list
  // holds the senders within the band's outer edge (the reference's edges in
  // a case without the fast test) and any motion triggers a rebuild. With a
  // skin s the list radius is rv = r_hi (1 + s), r_hi the band's outer
  // radius; a rebuild is due once some particle moved farther than
  // dmax = (rv - r_hi) / 2 less margins, so until then two particles within
  // the cutoff were within rv of each other at the last rebuild.
  const double skin = cfg.verlet_skin;
  for (int d = 0; d < 3; ++d) c.vrad[d] = c.rad[d];
  c.v_r2 = c.fast ? c.trim_r2 : INFINITY;
  c.v_dmax2 = 0.0f;
  if (c.fast && skin > 0.0) {
    const double r_hi = std::sqrt((double)c.trim_r2);
    const double rv = r_hi * (1.0 + skin);
    const double dmax = 0.5 * (rv - r_hi) - 4.0 * (double)c.trim_m;
    bool ok = dmax > 0.0;
    int vr[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
      if (c.nc[d] <= 1) continue;
      vr[d] = (int)std::ceil((rv + 2.0 * (double)c.trim_m) / (double)c.cell_size[d]);
      ok = ok && c.nc[d] >= 2 * vr[d] + 1;  // every cell visited once
    }
    if (ok) {
      for (int d = 0; d < 3; ++d) c.vrad[d] = vr[d];
      c.v_r2 = (float)(rv * rv);
      c.v_dmax2 = (float)(dmax * dmax);
    }
  }
  c.cell_off = (int)cell_off;
  c.p_off = (int)p_off;
  c.n = (int)in.n;
  c.cell_cap = INT_MAX;
  c.edge_cap = LLONG_MAX;
  c.cutoff_sq = cut * cut;
  // matscipy backend: the cutoff and box as the reference passes them to
  // matscipy (float64), distances in float64 (partition.py:393-395)
  c.f64_metric = cfg.nl_backend == SPH_NL_MATSCIPY;
  c.cut64_sq = in.r_cutoff * in.r_cutoff;
  for (int d = 0; d < 3; ++d) c.mat_box[d] = d < dim ? in.box[d] : 1.0;
  // kernels (kernel.py:51-103): sigma from the Python-float expressions
  const double ih = 1.0 / in.h;
  double sigma;
  if (cfg.kernel == SPH_KERNEL_QSK)
    sigma = dim == 2 ? 7.0 / 478.0 / M_PI * ih * ih : 3.0 / 359.0 / M_PI * ih * ih * ih;
  else
    sigma = dim == 2 ? 7.0 / 4.0 / M_PI * ih * ih : 21.0 / 16.0 / M_PI * ih * ih * ih;
  c.inv_h = (float)ih;
  c.sigma = (float)sigma;
  c.dsigma = (float)(-5.0 * sigma * ih);
  // integrator coefficients (integrator.py:26-30)
  c.dt = (float)(1.0 * in.dt);
  c.cv = (float)(in.tvf * 0.5 * in.dt);
  c.dt_rho = (float)in.dt_solver;
  c.dt64 = in.dt;
  for (int d = 0; d < 3; ++d) c.box64[d] = (double)c.box[d];
  // EOS (eos.py)
  c.eos = in.eos;
  c.p_ref = (float)in.p_ref;
  c.rho_ref = (float)in.rho_ref;
  c.p_bg = (float)in.p_bg;
  c.gamma = (float)in.gamma;
  c.inv_gamma = (float)(1.0 / in.gamma);
  c.rie_k = (float)(100.0 * in.u_ref * in.u_ref);
  if (in.eos == SPH_EOS_TAIT) {
    if (!(in.gamma > 0.0) || !(in.p_ref != 0.0) || !(in.rho_ref != 0.0)) {
      err = "invalid Tait EOS parameters";
      return -1;
    }
    c.p_bg_tvf = c.p_ref * (0.0f - 1.0f) + c.p_bg;
  } else {
    if (!(in.u_ref != 0.0)) {
      err = "invalid Riemann EOS parameters";
      return -1;
    }
    c.p_bg_tvf = c.rie_k * (0.0f - c.rho_ref) + c.p_bg;
  }
  c.c_ref = (float)in.c_ref;
  c.eta_limiter = (float)in.eta_limiter;
  // artificial_viscosity_fn_wrapper (solver.py:404-411)
  c.av_alpha = (float)in.artificial_alpha;
  c.av_hab = (float)in.dx;
  c.av_cab = 10.0f;
  c.av_eps = (float)(0.01 * in.dx * in.dx);
  // acceleration_delta_fn_wrapper(kernel, alpha, support = h, c_ref, rho_ref)
  // (solver.py:259-313, :682-689)
  c.delta_coef = (float)(in.diff_alpha * in.h * in.c_ref * in.rho_ref);
  // rho_evol_fn_delta_wrapper(delta, support = h, c_ref) (solver.py:33-105, :693)
  c.delta_rho_coef = (float)(in.c_ref * in.diff_delta * in.h);
  if (in.g_kind < SPH_GEXT_ZERO || in.g_kind > SPH_GEXT_REVERSE_X) {
    err = "unknown g_kind";
    return -1;
  }
  c.g_kind = in.g_kind;
  for (int d = 0; d < 3; ++d) {
    c.g[d] = (float)in.g[d];
    c.u_lid[d] = (float)in.u_lid[d];
  }
  c.g_lo = (float)in.g_band_lo;
  c.g_hi = (float)in.g_band_hi;
  if (in.bc_kind < SPH_BC_NONE || in.bc_kind > SPH_BC_HT) {
    err = "unknown bc_kind";
    return -1;
  }
  c.bc_kind = in.bc_kind;
  for (int k = 0; k < 2; ++k) {
    c.bc_T[k] = (float)in.bc_T[k];
    c.bc_x[k] = (float)in.bc_x[k];
  }
  return 0;
}

namespace {

int upload_cases(SphHandle* h, cudaStream_t st) {
  cudaError_t e = cudaMemcpyAsync(h->dc, h->hc.data(), sizeof(CaseDev) * h->n_cases,
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return cuda_check(e, "upload cases");
}

void drop_graph(SphHandle* h) {
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  if (h->gadv) cudaGraphExecDestroy(h->gadv);
  h->gexec = h->gadv = nullptr;
}

int launch_status(const char* what) { return cuda_check(cudaGetLastError(), what); }

// Sets the conditional of the rebuild node of a captured step from the flag
// the kick raised (and, for a drop-in step, the load's "positions differ from
// the binning" flag), and clears the flags.
__global__ void k_decide(unsigned* vflag, int nflags, unsigned long long* rebuilds,
                         cudaGraphConditionalHandle cond) {
  unsigned v = vflag[0];
  vflag[0] = 0u;
  if (nflags > 1) {
    v |= vflag[1];
    vflag[1] = 0u;
  }
  if (v) *rebuilds += 1ull;
  cudaGraphSetConditional(cond, v ? 1u : 0u);
}

// Rebuild: copy the state to the scratch set, sort it back into the resident
// set by cell (folding a pending forward result / bc_fn on the way, and
// keeping the positions as the new rebuild reference), then build the
// candidate lists. Stream-ordered and allocation-free (capturable).
int rebuild(SphHandle* h, cudaStream_t st, bool from_forward, bool apply_bc,
            bool lists = true) {
  LaunchCtx L = h->ctx(st);
  const Buffers& A = h->buf[0];
  const Buffers& B = h->buf[1];
  // the hashing kernel copies the resident set into the scratch set first
  launch_bin(L, B, A, h->R4, h->cellid, h->count, h->start, h->keyc, h->keys, h->tsrc, h->tkey,
             h->tcell, h->scan_tmp, h->C, false, from_forward, apply_bc, h->rref, &A);
  if (lists) launch_verlet(L, A, h->cellid, h->start);
  return launch_status("rebuild");
}

// Re-bin the current positions without moving them (neighbour-list
// allocate / update, a forward pass on a loaded state).
int bin_static(SphHandle* h, cudaStream_t st, bool lists = true) {
  int base = h->launch_count;
  int rc = rebuild(h, st, h->from_forward, h->pending_bc, lists);
  h->launch_count = base;
  h->binned = h->fresh = true;
  h->lists = lists;
  h->from_forward = false;
  h->pending_bc = false;
  return rc;
}

// One si_euler step (integrator.py:22-56), eagerly: kick-drift in place, a
// rebuild of the candidate lists when the kick found one due (the host reads
// the flag) or no lists exist yet, forward pass, bc_fn (applied to the
// accelerations in the force pass and folded into the state on the next read).
int step_once(SphHandle* h, cudaStream_t st) {
  h->launch_count = 0;
  LaunchCtx L = h->ctx(st);
  mark(L, 0);
  launch_kick(L, h->buf[0], h->R4, h->ref_cells, h->from_forward, h->pending_bc);
  mark(L, 5);
  bool rb = !h->lists;
  cudaError_t e = cudaSuccess;
  if (!rb) {
    unsigned v = 0;
    e = cudaMemcpyAsync(&v, h->vflag, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    rb = v != 0u;
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(h->vflag, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return cuda_check(e, "rebuild flag");
  mark(L, 6);
  if (rb) {
    const int base = h->launch_count;
    int rc = rebuild(h, st, false, false);
    if (rc) return rc;
    h->rebuild_launches = h->launch_count - base;
    h->launch_count = base;
    ++h->rebuilds_h;
  }
  mark(L, 1);
  launch_forward(L, h->buf[0], h->R4, h->R4, h->UT4, h->cellid, h->start, h->edgecnt, h->g_arr,
                 true, true);
  h->binned = h->lists = true;
  h->fresh = rb;
  h->from_forward = true;
  h->pending_bc = true;
  return launch_status("step");
}

bool steady(const SphHandle* h) { return h->lists && h->from_forward && h->pending_bc; }

// Capture one steady step: kick, decide, a conditional node whose body is the
// rebuild, forward pass. The rebuild runs on the device's own decision, so a
// replay never waits for the host. `advance`: the core of a drop-in step on a
// freshly loaded state instead -- kick (nothing pending to fold in), decide on
// both flags, rebuild; the caller launches the rest.
int capture_step(SphHandle* h, cudaStream_t st, bool advance = false) {
  h->launch_count = 0;
  LaunchCtx L = h->ctx(st);
  launch_kick(L, h->buf[0], h->R4, h->ref_cells, !advance, !advance);
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd);
  if (e != cudaSuccess) return cuda_check(e, "capture info");
  cudaGraphConditionalHandle cond;
  e = cudaGraphConditionalHandleCreate(&cond, g, 0u, 0u);
  if (e != cudaSuccess) return cuda_check(e, "conditional handle");
  k_decide<<<1, 1, 0, st>>>(h->vflag, advance ? 2 : 1, h->rebuilds_d, cond);
  count_launch(L);
  e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd);
  if (e != cudaSuccess) return cuda_check(e, "capture info");
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = cond;
  p.conditional.type = cudaGraphCondTypeIf;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &p);
  if (e != cudaSuccess) return cuda_check(e, "conditional node");
  e = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
  if (e != cudaSuccess) return cuda_check(e, "capture dependencies");
  cudaGraph_t body = p.conditional.phGraph_out[0];
  e = cudaStreamBeginCaptureToGraph(h->hs2, body, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_check(e, "capture rebuild");
  const int base = h->launch_count;
  int rc = rebuild(h, h->hs2, false, false);
  h->rebuild_launches = h->launch_count - base;
  h->launch_count = base;
  e = cudaStreamEndCapture(h->hs2, &body);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_check(e, "end rebuild capture");
  if (!advance)
    launch_forward(L, h->buf[0], h->R4, h->R4, h->UT4, h->cellid, h->start, h->edgecnt,
                   h->g_arr, true, true);
  return launch_status("step capture");
}

int capture_graph(SphHandle* h, bool advance = false) {
  cudaGraphExec_t& slot = advance ? h->gadv : h->gexec;
  if (slot) cudaGraphExecDestroy(slot);
  slot = nullptr;
  for (cudaStream_t* s : {&h->hs, &h->hs2}) {
    if (!*s) {
      cudaError_t e = cudaStreamCreateWithFlags(s, cudaStreamNonBlocking);
      if (e != cudaSuccess) return cuda_check(e, "stream create");
    }
  }
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(h->hs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_check(e, "begin capture");
  int rc = capture_step(h, h->hs, advance);
  e = cudaStreamEndCapture(h->hs, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cuda_check(e, "end capture");
  e = cudaGraphInstantiate(&slot, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_check(e, "graph instantiate");
  (advance ? h->gadv_g_arr : h->graph_g_arr) = h->g_arr;
  return 0;
}

}  // namespace

extern "C" {

int sph_abi_version(void) { return SPH_ABI_VERSION; }

const char* sph_last_error(void) { return g_last_error.c_str(); }

int sph_create(const SphConfig* cfg, const SphCase* cases, int32_t n_cases,
               SphHandle** out) try {
  if (!cfg || !cases || !out || n_cases <= 0)
    return fail((int)SPH_ERR_INVALID_ARG, "null argument or no cases");
  *out = nullptr;
  if (cfg->dim != 2 && cfg->dim != 3)
    return fail((int)SPH_ERR_INVALID_ARG, "Cell list spatial dimension must be 2 or 3");
  if (cfg->kernel != SPH_KERNEL_QSK && cfg->kernel != SPH_KERNEL_WC2K)
    return fail((int)SPH_ERR_INVALID_ARG, "kernel must be QSK or WC2K");
  if (cfg->nl_backend != SPH_NL_JAXMD && cfg->nl_backend != SPH_NL_MATSCIPY)
    return fail((int)SPH_ERR_INVALID_ARG, "nl_backend must be SPH_NL_JAXMD or SPH_NL_MATSCIPY");
  if (cfg->solver != SPH_SOLVER_SPH && cfg->solver != SPH_SOLVER_RIE &&
      cfg->solver != SPH_SOLVER_DELTA)
    return fail((int)SPH_ERR_INVALID_ARG, "solver must be SPH, RIE or DELTA");
  if (n_cases >= (1 << 26)) return fail((int)SPH_ERR_INVALID_ARG, "too many cases");
  if (!(cfg->verlet_skin >= 0.0 && cfg->verlet_skin <= 0.5))
    return fail((int)SPH_ERR_INVALID_ARG, "verlet_skin must lie in [0, 0.5]");
  SphHandle* h = new SphHandle();
  // frees the handle and its device buffers on every early return and on an
  // exception; released once the handle is complete
  struct Reclaim {
    SphHandle* h;
    ~Reclaim() {
      if (!h) return;
      for (void* p : h->allocs) cudaFree(p);
      delete h;
    }
  } reclaim{h};
  h->cfg = *cfg;
  h->n_cases = n_cases;
  h->cases.assign(cases, cases + n_cases);
  h->hc.resize(n_cases);
  std::vector<long long> off(n_cases + 1, 0);
  long long cells = 0, ref_cells = 0;
  for (int i = 0; i < n_cases; ++i) {
    if (cases[i].n <= 0)
      return fail((int)SPH_ERR_INVALID_ARG, "every case needs at least one particle");
    std::string err;
    if (make_case(*cfg, cases[i], off[i], cells, h->hc[i], err))
      return fail((int)SPH_ERR_INVALID_ARG, "case " + std::to_string(i) + ": " + err);
    h->hc[i].cref_off = (int)ref_cells;
    cells += h->hc[i].ncell + 1;  // + the parking cell of padding particles
    ref_cells += h->hc[i].ncref;
    off[i + 1] = off[i] + cases[i].n;
  }
  h->N = off[n_cases];
  h->lean = lean_config(*cfg, n_cases, h->hc[0]);
  h->C = cells;
  h->ref_cells = ref_cells;
  // Verlet slots: the candidates a particle of a case at lattice spacing dx
  // expects (sphere of the list radius over dx^d), times 1.5, plus 8
  {
    double est = 0.0;
    for (int i = 0; i < n_cases; ++i) {
      const CaseDev& c = h->hc[i];
      const double rv = c.fast ? std::sqrt((double)c.v_r2) : std::sqrt((double)c.cutoff_sq);
      const double q = cases[i].dx > 0.0 ? rv / cases[i].dx : 1e6;  // no spacing: most slots
      const double v = cfg->dim == 3 ? 4.0 / 3.0 * M_PI * q * q * q : M_PI * q * q;
      est = v > est ? v : est;
    }
    long long kv = (long long)std::ceil(1.5 * est) + 8;
    kv = (kv + 7) / 8 * 8;
    kv = kv < kVerletMinSlots ? kVerletMinSlots : (kv > kVerletMaxSlots ? kVerletMaxSlots : kv);
    h->kv = (int)kv;
  }
  if (h->N >= INT_MAX / 2 || h->C >= INT_MAX / 2)
    return fail((int)SPH_ERR_INVALID_ARG, "problem too large for 32-bit indices");
  const long long N = h->N;
  const bool need_nw = cfg->solver == SPH_SOLVER_RIE || cfg->is_free_slip;
  int rc = 0;
  for (int s = 0; s < 2 && !rc; ++s) {
    Buffers& b = h->buf[s];
    rc |= h->alloc(&b.P4, N) | h->alloc(&b.U4, N) | h->alloc(&b.V4, N) | h->alloc(&b.A4, N) |
          h->alloc(&b.A2, N) | h->alloc(&b.ETA, N) | h->alloc(&b.META, N) |
          h->alloc(&b.ORIG, N);
    if (need_nw) rc |= h->alloc(&b.NW4, N);
    if (cfg->fp64_positions) rc |= h->alloc(&b.RD, N);
    if (cfg->is_heat_conduction) rc |= h->alloc(&b.TH4, N);
  }
  if (!rc && cfg->is_heat_conduction) {
    rc |= h->alloc(&h->buf[0].TO, N);
    h->buf[1].TO = h->buf[0].TO;
  }
  if (!rc) {
    rc |= h->alloc(&h->R4, N) | h->alloc(&h->cellid, N);
    if (cfg->solver == SPH_SOLVER_RIE) rc |= h->alloc(&h->UT4, N);
    if (cfg->is_rho_evol && cfg->is_rho_renorm) rc |= h->alloc(&h->R4e, N);
    if (cfg->is_rho_evol && cfg->solver == SPH_SOLVER_DELTA)
      rc |= h->alloc(&h->dscr, 5 * (size_t)N);
    rc |= h->alloc(&h->count, h->C + 1) | h->alloc(&h->start, h->C + 1) |
          h->alloc(&h->keyc, N) | h->alloc(&h->keys, N) | h->alloc(&h->tsrc, N) |
          h->alloc(&h->tkey, N) | h->alloc(&h->tcell, N) | h->alloc(&h->rowcnt, N + 1) |
          h->alloc(&h->rowoff, N + 1) | h->alloc(&h->nbr, (size_t)h->kmax * N) |
          h->alloc(&h->nbr_cnt, N) | h->alloc(&h->vl, (size_t)h->kv * N) |
          h->alloc(&h->vcnt, N) | h->alloc(&h->rref, N) | h->alloc(&h->inv, N) |
          h->alloc(&h->cref_count, h->ref_cells + 1) | h->alloc(&h->vflag, 2) |
          h->alloc(&h->rebuilds_d, 1);
    long long m = h->C + 1 > N + 1 ? h->C + 1 : N + 1;
    rc |= h->alloc(&h->scan_tmp, scan_tmp_ints(m));
    rc |= h->alloc(&h->status, 1) | h->alloc(&h->edgecnt, n_cases) |
          h->alloc(&h->case_max, n_cases) | h->alloc(&h->dc, n_cases) |
          h->alloc(&h->case_off_d, n_cases + 1);
  }
  if (!rc) rc = cuda_check(cudaMemset(h->status, 0, sizeof(unsigned)), "memset");
  if (!rc) rc = cuda_check(cudaMemset(h->vflag, 0, 2 * sizeof(unsigned)), "memset");
  if (!rc) rc = cuda_check(cudaMemset(h->rebuilds_d, 0, sizeof(unsigned long long)), "memset");
  if (!rc) rc = cuda_check(cudaMemset(h->rref, 0, sizeof(float4) * N), "memset");
  if (!rc) rc = cuda_check(prepare_kernels(h->kv), "kernel attributes");
  if (!rc)
    rc = cuda_check(cudaMemcpy(h->case_off_d, off.data(), sizeof(long long) * (n_cases + 1),
                               cudaMemcpyHostToDevice),
                    "upload offsets");
  if (!rc) rc = upload_cases(h, 0);
  if (rc) return rc;
  reclaim.h = nullptr;
  *out = h;
  return 0;
} catch (...) {
  return host_error();
}

int sph_destroy(SphHandle* h) try {
  if (!h) return 0;
  drop_graph(h);
  for (int k = 0; k < SphHandle::kCopyStreams; ++k) {
    if (h->cs[k]) cudaStreamDestroy(h->cs[k]);
    if (h->join[k]) cudaEventDestroy(h->join[k]);
  }
  if (h->fork) cudaEventDestroy(h->fork);
  if (h->hs) cudaStreamDestroy(h->hs);
  if (h->hs2) cudaStreamDestroy(h->hs2);
  for (void* p : h->allocs) cudaFree(p);
  cudaFree(h->layer_pts);
  cudaFree(h->layer_start);
  delete h;
  return 0;
} catch (...) {
  return host_error();
}

int sph_update_cases(SphHandle* h, const SphCase* cases, int32_t n_cases) try {
  if (!h || !cases) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  if (n_cases != h->n_cases) return fail((int)SPH_ERR_INVALID_ARG, "case count changed");
  std::vector<CaseDev> next(n_cases);
  for (int i = 0; i < n_cases; ++i) {
    const SphCase& a = h->cases[i];
    const SphCase& b = cases[i];
    bool same = a.n == b.n && a.r_cutoff == b.r_cutoff;
    for (int d = 0; d < 3; ++d) same = same && a.box[d] == b.box[d];
    if (!same) return fail((int)SPH_ERR_INVALID_ARG, "particle count, box or cutoff changed");
    std::string err;
    if (make_case(h->cfg, b, h->hc[i].p_off, h->hc[i].cell_off, next[i], err))
      return fail((int)SPH_ERR_INVALID_ARG, "case " + std::to_string(i) + ": " + err);
    next[i].cell_cap = h->hc[i].cell_cap;
    next[i].edge_cap = h->hc[i].edge_cap;
    next[i].cref_off = h->hc[i].cref_off;
  }
  h->cases.assign(cases, cases + n_cases);
  h->hc = next;
  const int lean = lean_config(h->cfg, n_cases, h->hc[0]);
  if (lean != h->lean) {
    // the list format changes with the passes: the lists must be rebuilt
    h->lean = lean;
    h->lists = false;
  }
  drop_graph(h);
  return upload_cases(h, 0);
} catch (...) {
  return host_error();
}

int sph_set_state(SphHandle* h, const SphStateView* s, void* stream) try {
  if (!h || !s) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  if (s->n != h->N) return fail((int)SPH_ERR_INVALID_ARG, "state has the wrong particle count");
  if (!s->r || !s->tag || !s->u || !s->v || !s->dudt || !s->dvdt || !s->rho || !s->p ||
      !s->mass || !s->eta)
    return fail((int)SPH_ERR_INVALID_ARG, "missing state field");
  if (h->buf[0].NW4 && !s->nw)
    return fail((int)SPH_ERR_INVALID_ARG, "wall normals nw are required by this solver");
  if (h->buf[0].TH4 && (!s->T || !s->dTdt || !s->kappa || !s->Cp))
    return fail((int)SPH_ERR_INVALID_ARG, "heat conduction needs T, dTdt, kappa and Cp");
  bool garr = false;
  for (const auto& c : h->hc) garr |= c.g_kind == SPH_GEXT_ARRAY;
  if (garr && !s->g_ext)
    return fail((int)SPH_ERR_INVALID_ARG, "g_ext array required by SPH_GEXT_ARRAY");
  cudaStream_t st = (cudaStream_t)stream;
  cudaMemsetAsync(h->status, 0, sizeof(unsigned), st);  // a new state starts clean
  launch_pack(h->ctx(st), *s, h->buf[0], h->case_off_d);
  h->g_arr = s->g_ext;
  h->has_state = true;
  h->binned = h->lists = h->fresh = h->from_forward = h->pending_bc = false;
  return launch_status("set_state");
} catch (...) {
  return host_error();
}

int sph_get_state(SphHandle* h, SphStateView* s, void* stream) try {
  if (!h || !s) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  if (s->n != h->N) return fail((int)SPH_ERR_INVALID_ARG, "state has the wrong particle count");
  if (!s->r || !s->u || !s->v || !s->dudt || !s->dvdt || !s->rho || !s->p)
    return fail((int)SPH_ERR_INVALID_ARG, "missing state field");
  // after a binning the read-back runs per original index (coalesced writes)
  launch_unpack(h->ctx((cudaStream_t)stream), h->buf[0], h->R4, *s, h->from_forward,
                h->pending_bc, nullptr, 0.f, h->binned ? h->inv : nullptr);
  return launch_status("get_state");
} catch (...) {
  return host_error();
}

int sph_nl_update(SphHandle* h, void* stream) try {
  if (!h) return fail((int)SPH_ERR_INVALID_ARG, "null handle");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  return bin_static(h, (cudaStream_t)stream);
} catch (...) {
  return host_error();
}

int sph_nl_allocate(SphHandle* h, int64_t extra_capacity, SphNLCapacity* cap_out,
                    void* stream) try {
  if (!h) return fail((int)SPH_ERR_INVALID_ARG, "null handle");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  cudaStream_t st = (cudaStream_t)stream;
  // allocation sizes the capacities from the data and never flags an overflow
  for (auto& c : h->hc) {
    c.cell_cap = INT_MAX;
    c.edge_cap = LLONG_MAX;
  }
  int rc = upload_cases(h, st);
  if (!rc) rc = bin_static(h, st, false);  // the capacities need no candidate lists
  if (rc) return rc;
  LaunchCtx L = h->ctx(st);
  launch_row_counts(L, h->buf[0], h->cellid, h->start, h->rowcnt);
  launch_alloc_stats(L, h->buf[0], h->cellid, h->start, h->rowcnt, h->case_max, h->edgecnt);
  if ((rc = launch_status("allocate stats"))) return rc;
  std::vector<int> maxocc_c(h->n_cases);
  std::vector<unsigned long long> occ_c(h->n_cases);
  cudaError_t e = cudaMemcpyAsync(maxocc_c.data(), h->case_max, sizeof(int) * h->n_cases,
                                  cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(occ_c.data(), h->edgecnt, sizeof(unsigned long long) * h->n_cases,
                        cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if ((rc = cuda_check(e, "allocate readback"))) return rc;
  const double mult = h->cfg.capacity_multiplier;
  const int nb = h->cfg.dim == 3 ? 27 : 9;
  for (int i = 0; i < h->n_cases; ++i) {
    CaseDev& c = h->hc[i];
    const long long maxocc = maxocc_c[i], occ = (long long)occ_c[i];
    // _estimate_cell_capacity (jax_md/partition.py:195-199) + extra capacity
    c.cell_cap = (int)(maxocc * mult) + (int)extra_capacity;
    // max_occupancy = int(occupancy * multiplier + N * extra) (:956-971)
    long long mo = (long long)((float)occ * (float)mult + (float)(c.n * extra_capacity));
    long long n = c.n;
    long long cand = c.use_cells ? n * nb * (long long)c.cell_cap : n * n;
    long long limit = h->cfg.mask_self ? n * (n - 1) : n * n;
    if (mo > cand) mo = cand;
    if (mo > limit) mo = limit;
    c.edge_cap = mo;
    if (i == 0 && cap_out) {
      cap_out->cell_capacity = c.cell_cap;
      cap_out->max_occupancy = mo;
      cap_out->occupancy = occ;
      cap_out->max_cell_occupancy = maxocc;
    }
  }
  // the captured step reads the capacities from device memory: no re-capture
  return upload_cases(h, st);
} catch (...) {
  return host_error();
}

int sph_nl_set_capacity(SphHandle* h, const SphNLCapacity* cap) try {
  if (!h || !cap) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  if (cap->cell_capacity < 0 || cap->cell_capacity > INT_MAX || cap->max_occupancy < 0)
    return fail((int)SPH_ERR_INVALID_ARG, "capacity out of range");
  bool same = true;
  for (const auto& c : h->hc)
    same = same && c.cell_cap == (int)cap->cell_capacity && c.edge_cap == cap->max_occupancy;
  if (same) return 0;  // nothing to upload (a drop-in step sets them on every call)
  for (auto& c : h->hc) {
    c.cell_cap = (int)cap->cell_capacity;
    c.edge_cap = cap->max_occupancy;
  }
  return upload_cases(h, 0);
} catch (...) {
  return host_error();
}

int sph_nl_edges(SphHandle* h, int32_t* idx, int64_t capacity, int64_t* count_dev,
                 void* stream) try {
  if (!h || !idx || !count_dev || capacity < 0)
    return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  if (!h->binned) return fail((int)SPH_ERR_INVALID_ARG, "neighbour list not built");
  // the edges come from a binning of the current positions
  if (!h->fresh) {
    int rc = bin_static(h, (cudaStream_t)stream, h->lists);
    if (rc) return rc;
  }
  LaunchCtx L = h->ctx((cudaStream_t)stream);
  launch_edges(L, h->buf[0], h->cellid, h->start, h->rowcnt, h->rowoff, h->scan_tmp, idx,
               capacity, (long long*)count_dev);
  return launch_status("edges");
} catch (...) {
  return host_error();
}

int sph_forward(SphHandle* h, void* stream) try {
  if (!h) return fail((int)SPH_ERR_INVALID_ARG, "null handle");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = 0;
  if (!h->lists || h->from_forward) rc = bin_static(h, st);
  if (rc) return rc;
  launch_forward(h->ctx(st), h->buf[0], h->R4, h->R4, h->UT4, h->cellid, h->start,
                 h->edgecnt, h->g_arr, false, true);
  h->from_forward = true;
  h->pending_bc = false;
  return launch_status("forward");
} catch (...) {
  return host_error();
}

int sph_step(SphHandle* h, int32_t nsteps, void* stream) try {
  if (!h) return fail((int)SPH_ERR_INVALID_ARG, "null handle");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  if (nsteps < 0) return fail((int)SPH_ERR_INVALID_ARG, "negative step count");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = 0;
  // the first step after loading a state runs eagerly (it folds the loaded
  // state in and builds the first candidate lists); every later step replays
  // the captured steady step
  if (nsteps > 0 && !steady(h)) {
    if ((rc = step_once(h, st))) return rc;
    --nsteps;
  }
  if (h->graph_g_arr != h->g_arr) drop_graph(h);
  while (nsteps > 0) {
    if (!h->gexec && (rc = capture_graph(h))) return rc;
    if ((rc = cuda_check(cudaGraphLaunch(h->gexec, st), "graph launch"))) return rc;
    h->fresh = false;
    --nsteps;
  }
  return 0;
} catch (...) {
  return host_error();
}

}  // extern "C"

namespace {
// Where a caller array lives: device memory (used in place) or pinned
// (page-locked) host memory (copied by DMA to and from a device staging
// slot). Anything else -- pageable memory -- is rejected before any work.
int pinned_host(const void* p, const char* name, bool* host, void** mapped = nullptr) {
  *host = false;
  if (mapped) *mapped = nullptr;
  if (!p) return 0;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail((int)SPH_ERR_INVALID_ARG, std::string(name) + ": unknown pointer");
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return 0;
  if (a.type == cudaMemoryTypeHost) {
    *host = true;
    if (mapped) *mapped = a.devicePointer;
    return 0;
  }
  return fail((int)SPH_ERR_INVALID_ARG,
              std::string(name) + ": host arrays must be pinned (page-locked) memory");
}

// The device arrays a steady handle carries from one step to the next: the
// resident particle set, the pending forward result, the binning (cells,
// starts, inverse permutation), the rebuild reference positions and the
// candidate lists. Everything else is rebuilt or reset inside a step.
std::vector<std::pair<void*, size_t>> carried_state(const SphHandle* h) {
  const size_t N = (size_t)h->N;
  const Buffers& b = h->buf[0];
  std::vector<std::pair<void*, size_t>> r = {
      {b.P4, sizeof(float4) * N},   {b.U4, sizeof(float4) * N},
      {b.V4, sizeof(float4) * N},   {b.A4, sizeof(float4) * N},
      {b.A2, sizeof(float4) * N},   {b.ETA, sizeof(float) * N},
      {b.META, sizeof(int) * N},    {b.ORIG, sizeof(int) * N},
      {h->R4, sizeof(float4) * N},  {h->cellid, sizeof(int) * N},
      {h->start, sizeof(int) * ((size_t)h->C + 1)}, {h->rref, sizeof(float4) * N},
      {h->vl, sizeof(int) * (size_t)h->kv * N},     {h->vcnt, sizeof(int) * N},
      {h->inv, sizeof(int) * N}};
  if (b.NW4) r.push_back({b.NW4, sizeof(float4) * N});
  if (b.RD) r.push_back({b.RD, sizeof(double4_32a) * N});
  return r;
}

int snap_copy(SphHandle* h, int slot, bool save, cudaStream_t st) {
  size_t off = (size_t)slot * h->snap_stride;
  for (const auto& reg : carried_state(h)) {
    unsigned char* dst = h->snap + off;
    cudaError_t e = save ? cudaMemcpyAsync(dst, reg.first, reg.second, cudaMemcpyDeviceToDevice, st)
                         : cudaMemcpyAsync(reg.first, dst, reg.second, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_check(e, "snapshot copy");
    off += (reg.second + 255) & ~size_t(255);
  }
  return 0;
}

}  // namespace

extern "C" {

int sph_advance(SphHandle* h, const SphStateView* in_, SphStateView* out_, const float* ref_r_,
                float threshold_sq, uint32_t* status_dev, void* stream) try {
  if (!h || !in_ || !out_ || !status_dev) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  SphStateView vin = *in_, vout = *out_;
  const SphStateView* in = &vin;
  SphStateView* out = &vout;
  cudaStream_t st = (cudaStream_t)stream;
  // fields in pinned host memory go through device staging slots: one DMA
  // copy per field in, one per result field out
  const size_t N = (size_t)h->N;
  const size_t vec = sizeof(float) * (size_t)h->cfg.dim * N, sc = sizeof(float) * N;
  struct Field {
    const char* name;
    void** in;
    void** out;
    size_t bytes;
  };
  Field fields[] = {
      {"r", (void**)&vin.r, (void**)&vout.r, vec},
      {"tag", (void**)&vin.tag, nullptr, sizeof(int32_t) * N},
      {"u", (void**)&vin.u, (void**)&vout.u, vec},
      {"v", (void**)&vin.v, (void**)&vout.v, vec},
      {"dudt", (void**)&vin.dudt, (void**)&vout.dudt, vec},
      {"dvdt", (void**)&vin.dvdt, (void**)&vout.dvdt, vec},
      {"drhodt", (void**)&vin.drhodt, (void**)&vout.drhodt, sc},
      {"rho", (void**)&vin.rho, (void**)&vout.rho, sc},
      {"p", (void**)&vin.p, (void**)&vout.p, sc},
      {"mass", (void**)&vin.mass, nullptr, sc},
      {"eta", (void**)&vin.eta, nullptr, sc},
      {"nw", (void**)&vin.nw, (void**)&vout.nw, vec},  // out: recomputed normals
      {"g_ext", (void**)&vin.g_ext, nullptr, vec},
      {"T", (void**)&vin.T, (void**)&vout.T, sc},
      {"dTdt", (void**)&vin.dTdt, (void**)&vout.dTdt, sc},
      {"kappa", (void**)&vin.kappa, nullptr, sc},
      {"Cp", (void**)&vin.Cp, nullptr, sc},
  };
  constexpr int kFields = sizeof(fields) / sizeof(fields[0]);
  // inputs the step never reads: v (the kick sets v = u + tvf dt/2 dvdt
  // before anything reads it, integrator.py:26-27), the old pressure (read by
  // the Riemann continuity only) and drho/dt (carried over by a summation,
  // when asked for); they are neither copied nor loaded
  const bool rie_evol = h->cfg.solver == SPH_SOLVER_RIE && h->cfg.is_rho_evol;
  if (!in_->v || !in_->p) return fail((int)SPH_ERR_INVALID_ARG, "missing state field");
  vin.v = nullptr;
  if (!rie_evol) vin.p = nullptr;
  const bool drhodt_unread = h->cfg.is_rho_evol || !vout.drhodt;
  if (drhodt_unread) vin.drhodt = nullptr;
  bool hin[kFields], hout[kFields], href = false, hst = false;
  bool any = false;
  for (int k = 0; k < kFields; ++k) {
    void* mapped = nullptr;
    int rc = pinned_host(*fields[k].in, fields[k].name, &hin[k], &mapped);
    hout[k] = false;
    if (!rc && fields[k].out) rc = pinned_host(*fields[k].out, fields[k].name, &hout[k]);
    if (rc) return rc;
    // a mapped host input is read by the load kernel straight over the host
    // link (coalesced; measured faster than a staging copy); results go back
    // by DMA from staging (measured faster than writes over the link)
    if (hin[k] && mapped) {
      *fields[k].in = mapped;
      hin[k] = false;
    }
    any = any || hin[k] || hout[k];
  }
  int vrc = pinned_host(ref_r_, "ref_r", &href);
  if (!vrc) vrc = pinned_host(status_dev, "status", &hst);
  if (vrc) return vrc;
  any = any || href;
  if (any && !h->stage) {  // allocated once, on the first call with host arrays
    h->stage_slot = (vec + 255) / 256 * 256;
    if (h->alloc(&h->stage, h->stage_slot * (kFields + 1))) return SPH_ERR_CUDA;
    cudaError_t e0 = cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming);
    for (int k = 0; k < SphHandle::kCopyStreams && e0 == cudaSuccess; ++k) {
      e0 = cudaStreamCreateWithFlags(&h->cs[k], cudaStreamNonBlocking);
      if (e0 == cudaSuccess) e0 = cudaEventCreateWithFlags(&h->join[k], cudaEventDisableTiming);
    }
    if (e0 != cudaSuccess) return cuda_check(e0, "copy streams");
  }
  // fork: the copy streams start after the work already on `st`; join: `st`
  // continues after all of them
  auto fork = [&]() {
    cudaError_t r = cudaEventRecord(h->fork, st);
    for (int k = 0; k < SphHandle::kCopyStreams && r == cudaSuccess; ++k)
      r = cudaStreamWaitEvent(h->cs[k], h->fork, 0);
    return r;
  };
  auto join = [&]() {
    cudaError_t r = cudaSuccess;
    for (int k = 0; k < SphHandle::kCopyStreams && r == cudaSuccess; ++k) {
      r = cudaEventRecord(h->join[k], h->cs[k]);
      if (r == cudaSuccess) r = cudaStreamWaitEvent(st, h->join[k], 0);
    }
    return r;
  };
  cudaError_t e = any ? fork() : cudaSuccess;
  int ncopy = 0;
  void* host_dst[kFields] = {};
  for (int k = 0; k < kFields; ++k) {
    void* slot = h->stage ? h->stage + h->stage_slot * k : nullptr;
    if (hin[k]) {
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(slot, *fields[k].in, fields[k].bytes, cudaMemcpyHostToDevice,
                            h->cs[ncopy++ % SphHandle::kCopyStreams]);
      *fields[k].in = slot;
    }
    if (hout[k]) {  // the result goes to the slot, then to the host array
      host_dst[k] = *fields[k].out;
      *fields[k].out = slot;
    }
  }
  const float* ref_r = ref_r_;
  if (href) {
    void* slot = h->stage + h->stage_slot * kFields;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(slot, ref_r_, vec, cudaMemcpyHostToDevice,
                          h->cs[ncopy++ % SphHandle::kCopyStreams]);
    ref_r = (const float*)slot;
  }
  if (any && e == cudaSuccess) e = join();
  if (e != cudaSuccess) return cuda_check(e, "advance input copy");
  if (in->n != h->N || out->n != h->N)
    return fail((int)SPH_ERR_INVALID_ARG, "state has the wrong particle count");
  if (!h->cfg.is_rho_evol && out_->drhodt && !in_->drhodt)
    return fail((int)SPH_ERR_INVALID_ARG, "missing state field");
  if (!in->r || !in->tag || !in->u || !in->dudt || !in->dvdt || !in->rho ||
      !in->mass || !in->eta || !out->r || !out->u || !out->v || !out->dudt || !out->dvdt ||
      !out->rho || !out->p)
    return fail((int)SPH_ERR_INVALID_ARG, "missing state field");
  if (h->buf[0].NW4 && !in->nw)
    return fail((int)SPH_ERR_INVALID_ARG, "wall normals nw are required by this solver");
  if (h->buf[0].TH4 &&
      (!in->T || !in->dTdt || !in->kappa || !in->Cp || !out->T || !out->dTdt))
    return fail((int)SPH_ERR_INVALID_ARG, "heat conduction needs T, dTdt, kappa and Cp");
  bool garr = false;
  for (const auto& c : h->hc) garr |= c.g_kind == SPH_GEXT_ARRAY;
  if (garr && !in->g_ext)
    return fail((int)SPH_ERR_INVALID_ARG, "g_ext array required by SPH_GEXT_ARRAY");
  LaunchCtx L = h->ctx(st);
  const Buffers& A = h->buf[0];
  const Buffers& B = h->buf[1];
  e = cudaMemsetAsync(h->status, 0, sizeof(unsigned), st);
  h->g_arr = in->g_ext;
  h->launch_count = 0;
  if (h->binned) {
    // warm: the state goes to the sorted slots of the binning the handle
    // holds; when no position differs from the one there (the caller passed
    // back the last result) the binning and candidate lists still fit, and
    // only the skin test decides on a rebuild -- the host reads both flags
    if (e == cudaSuccess) e = cudaMemsetAsync(h->vflag, 0, 2 * sizeof(unsigned), st);
    launch_pack(L, *in, A, h->case_off_d, h->inv, h->vflag + 1);
    if (h->lists) {
      // kick, then a rebuild if the kick or the load asked for one: decided
      // on the device inside a captured graph, no host round trip
      if (h->gadv && h->gadv_g_arr != h->g_arr) {
        cudaGraphExecDestroy(h->gadv);
        h->gadv = nullptr;
      }
      int rc = 0;
      if (!h->gadv && (rc = capture_graph(h, true))) return rc;
      if (e == cudaSuccess) e = cudaGraphLaunch(h->gadv, st);
    } else {
      launch_kick(L, A, h->R4, h->ref_cells, false, false);
      int rc = rebuild(h, st, false, false);
      if (rc) return rc;
      ++h->rebuilds_h;
      if (e == cudaSuccess) e = cudaMemsetAsync(h->vflag, 0, 2 * sizeof(unsigned), st);
    }
    if (e != cudaSuccess) return cuda_check(e, "advance core");
  } else {
    // cold: load into the scratch set, kick there, sort into the resident
    // set (the rebuild needs no copy)
    launch_pack(L, *in, B, h->case_off_d);
    launch_kick(L, B, h->R4, h->ref_cells, false, false);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->vflag, 0, sizeof(unsigned), st);
    launch_bin(L, B, A, h->R4, h->cellid, h->count, h->start, h->keyc, h->keys, h->tsrc,
               h->tkey, h->tcell, h->scan_tmp, h->C, false, false, false, h->rref);
    launch_verlet(L, A, h->cellid, h->start);
    ++h->rebuilds_h;
  }
  bool any_out = false;
  for (int k = 0; k < kFields; ++k) any_out = any_out || host_dst[k];
  // copy the result fields in `mask` (bit k: fields[k]) back to host memory
  ncopy = 0;
  auto copy_back = [&](unsigned mask) {
    if (!any_out) return;  // device outputs: the unpack wrote them in place
    if (e == cudaSuccess) e = fork();
    for (int k = 0; k < kFields; ++k)
      if ((mask >> k & 1u) && host_dst[k] && e == cudaSuccess)
        e = cudaMemcpyAsync(host_dst[k], h->stage + h->stage_slot * k, fields[k].bytes,
                            cudaMemcpyDeviceToHost, h->cs[ncopy++ % SphHandle::kCopyStreams]);
  };
  constexpr unsigned kRUV = 1u << 0 | 1u << 2 | 1u << 3 | 1u << 11,  // with nw
                     kRhoP = 1u << 7 | 1u << 8 | 1u << 13 | 1u << 14,  // with T, dTdt
                     kRates = 1u << 4 | 1u << 5 | 1u << 6;
  // r, u and v are final after the kick unless the wall BC pass of the SPH
  // and DELTA solvers rewrites wall velocities: then they go back to host
  // memory while the forward pass runs (fields 0..3 of the list: r, tag, u, v)
  const bool early = any_out && !(h->cfg.is_bc_trick && h->cfg.solver != SPH_SOLVER_RIE);
  if (early) {
    SphStateView first{};
    first.n = out->n;
    first.r = out->r;
    first.u = out->u;
    first.v = out->v;
    first.nw = out->nw;
    launch_unpack(L, A, h->R4, first, false, true, ref_r, threshold_sq, h->inv);
    copy_back(kRUV);
    out->r = out->u = out->v = out->nw = nullptr;
    ref_r = nullptr;
  }
  // density passes and wall BC: rho and p (and r, u, v, when the wall BC
  // rewrote wall velocities) are final and go back while the force pass runs
  launch_forward(L, A, h->R4, h->R4, h->UT4, h->cellid, h->start, h->edgecnt, h->g_arr, true,
                 true, 1);
  {
    SphStateView mid{};
    mid.n = out->n;
    mid.rho = out->rho;
    mid.p = out->p;
    mid.r = out->r;
    mid.u = out->u;
    mid.v = out->v;
    mid.T = out->T;
    mid.dTdt = out->dTdt;
    mid.nw = out->nw;
    launch_unpack(L, A, h->R4, mid, true, true, ref_r, threshold_sq, h->inv);
    copy_back(kRhoP | (early ? 0u : kRUV));
    out->rho = out->p = out->r = out->u = out->v = out->T = out->dTdt = out->nw = nullptr;
    ref_r = nullptr;
  }
  launch_forward(L, A, h->R4, h->R4, h->UT4, h->cellid, h->start, h->edgecnt, h->g_arr, true,
                 true, 2);
  launch_unpack(L, A, h->R4, *out, true, true, nullptr, threshold_sq, h->inv);
  if (any_out) {
    copy_back(kRates);
    if (e == cudaSuccess) e = join();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(status_dev, h->status, sizeof(unsigned),
                        hst ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->status, 0, sizeof(unsigned), st);
  h->has_state = h->binned = h->lists = true;
  h->fresh = false;  // the binning may predate the kick
  h->from_forward = h->pending_bc = true;
  // results in host memory: return once they are there
  if (e == cudaSuccess && (any_out || hst)) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_check(e, "advance");
  return launch_status("advance");
} catch (...) {
  return host_error();
}

int sph_set_wall_layer(SphHandle* h, const float* layer, int64_t m, const double* offset,
                       double cutoff) try {
  if (!h) return fail((int)SPH_ERR_INVALID_ARG, "null handle");
  if (m < 0 || (m > 0 && (!layer || !offset || !(cutoff > 0.0))))
    return fail((int)SPH_ERR_INVALID_ARG, "bad wall layer");
  if (m > INT_MAX / 2) return fail((int)SPH_ERR_INVALID_ARG, "wall layer too large");
  if (m > 0 && h->n_cases != 1)
    return fail((int)SPH_ERR_INVALID_ARG, "a wall layer needs a single-case handle");
  if (m > 0 && !h->buf[0].NW4)
    return fail((int)SPH_ERR_INVALID_ARG,
                "wall normals are kept only by the Riemann solver or with free slip");
  cudaFree(h->layer_pts);
  cudaFree(h->layer_start);
  h->layer_pts = nullptr;
  h->layer_start = nullptr;
  h->layer = WallLayer{};
  drop_graph(h);  // the kick of a captured step carries the layer
  if (m == 0) return 0;
  const int dim = h->cfg.dim;
  const CaseDev& c = h->hc[0];
  WallLayer w{};
  w.n = (int)m;
  // cells at least one search radius wide, so the 3^d cells around a point
  // hold its radius; the grid is coarsened (widest side halved) until it has
  // no more cells than about four per layer point -- any such grid finds the
  // same nearest point
  long long n[3];
  for (int d = 0; d < 3; ++d) {
    const double q = d < dim ? std::floor((double)c.box[d] / cutoff) : 1.0;
    n[d] = q < 1.0 ? 1 : (q > 1048576.0 ? 1048576 : (long long)q);
  }
  while (n[0] * n[1] * n[2] > 4 * m + 64) {
    const int d = n[0] >= n[1] && n[0] >= n[2] ? 0 : (n[1] >= n[2] ? 1 : 2);
    n[d] = (n[d] + 1) / 2;
  }
  for (int d = 0; d < 3; ++d) {
    const double box = d < dim ? (double)c.box[d] : 1.0;
    w.nc[d] = (int)n[d];
    w.cs[d] = (float)(box / n[d]);
    w.off[d] = d < dim ? (float)offset[d] : 0.f;
  }
  w.cut2 = (float)(cutoff * cutoff);
  // counting sort of the points by cell (stable: ascending index in a cell)
  const long long ncell = (long long)w.nc[0] * w.nc[1] * w.nc[2];
  std::vector<int> cell(m), start(ncell + 1, 0);
  for (int64_t k = 0; k < m; ++k) {
    int ci[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
      const double box = c.box[d];
      double x = layer[k * dim + d];
      x -= box * std::floor(x / box);
      int q = (int)(x / w.cs[d]);
      ci[d] = q < 0 ? 0 : (q >= w.nc[d] ? w.nc[d] - 1 : q);
    }
    cell[k] = ci[0] + w.nc[0] * (ci[1] + w.nc[1] * ci[2]);
    ++start[cell[k] + 1];
  }
  for (long long q = 0; q < ncell; ++q) start[q + 1] += start[q];
  std::vector<int> fill(start.begin(), start.end() - 1);
  std::vector<float4> pts(m);
  for (int64_t k = 0; k < m; ++k) {
    float4 p = make_float4(layer[k * dim], layer[k * dim + 1], dim == 3 ? layer[k * dim + 2] : 0.f,
                           0.f);
    int idx = (int)k;
    std::memcpy(&p.w, &idx, sizeof(int));
    pts[fill[cell[k]]++] = p;
  }
  cudaError_t e = cudaMalloc(&h->layer_pts, sizeof(float4) * m);
  if (e == cudaSuccess) e = cudaMalloc(&h->layer_start, sizeof(int) * (ncell + 1));
  if (e == cudaSuccess)
    e = cudaMemcpy(h->layer_pts, pts.data(), sizeof(float4) * m, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(h->layer_start, start.data(), sizeof(int) * (ncell + 1),
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_check(e, "wall layer upload");
  w.pts = h->layer_pts;
  w.start = h->layer_start;
  h->layer = w;
  return 0;
} catch (...) {
  return host_error();
}

int sph_set_block_size(SphHandle* h, int32_t threads) try {
  if (!h) return fail((int)SPH_ERR_INVALID_ARG, "null handle");
  if (threads < 32 || threads > 256 || threads % 32)
    return fail((int)SPH_ERR_INVALID_ARG, "block size must be a multiple of 32 in [32, 256]");
  h->block = threads;
  drop_graph(h);
  return 0;
} catch (...) {
  return host_error();
}

int sph_set_force_variant(SphHandle* h, int32_t variant) try {
  if (!h) return fail((int)SPH_ERR_INVALID_ARG, "null handle");
  if (variant != SPH_FORCE_GATHER && variant != SPH_FORCE_STAGED)
    return fail((int)SPH_ERR_INVALID_ARG, "variant must be SPH_FORCE_GATHER or SPH_FORCE_STAGED");
  h->force_variant = variant;
  drop_graph(h);
  return 0;
} catch (...) {
  return host_error();
}

int sph_step_launch_count(SphHandle* h, int32_t* count) try {
  if (!h || !count) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  *count = h->launch_count;
  return 0;
} catch (...) {
  return host_error();
}

int sph_list_format(SphHandle* h, int32_t* format) try {
  if (!h || !format) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  *format = h->lean;
  return 0;
} catch (...) {
  return host_error();
}

int sph_profile_step(SphHandle* h, int32_t nsteps, float* ms, void* stream) try {
  if (!h || !ms || nsteps <= 0) return fail((int)SPH_ERR_INVALID_ARG, "bad argument");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  cudaStream_t st = (cudaStream_t)stream;
  // events: 0 step start, 5 kick end, 6 rebuild start (after the host read
  // the flag), 1 rebuild end, 2 density end, 3 wall end, 4 force end
  cudaEvent_t ev[7] = {};
  int rc = 0;
  for (int k = 0; k < 7 && !rc; ++k) rc = cuda_check(cudaEventCreate(&ev[k]), "profile events");
  for (int k = 0; k < 6; ++k) ms[k] = 0.f;
  for (int i = 0; i < nsteps && !rc; ++i) {
    h->ev = ev;
    rc = step_once(h, st);
    h->ev = nullptr;
    if (rc) break;
    cudaError_t e = cudaEventSynchronize(ev[4]);
    if ((rc = cuda_check(e, "profile sync"))) break;
    float t = 0.f, t2 = 0.f;
    cudaEventElapsedTime(&t, ev[0], ev[5]);
    cudaEventElapsedTime(&t2, ev[6], ev[1]);
    ms[0] += (t + t2) / nsteps;  // kick + rebuild, without the host's read
    ms[4] += t / nsteps;
    ms[5] += t2 / nsteps;
    for (int k = 1; k < 4; ++k) {
      cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
      ms[k] += t / nsteps;
    }
  }
  for (int k = 0; k < 7; ++k)
    if (ev[k]) cudaEventDestroy(ev[k]);
  return rc;
} catch (...) {
  return host_error();
}

int sph_snapshot_init(SphHandle* h, int32_t slots) try {
  if (!h || slots <= 0) return fail((int)SPH_ERR_INVALID_ARG, "bad argument");
  if (h->snap_slots) return fail((int)SPH_ERR_INVALID_ARG, "snapshots already initialised");
  const SphConfig& c = h->cfg;
  if (c.solver != SPH_SOLVER_SPH || c.is_rho_evol || c.is_heat_conduction)
    return fail((int)SPH_ERR_INVALID_ARG,
                "snapshots cover the SPH solver with density summation, no heat conduction");
  size_t stride = 0;
  for (const auto& reg : carried_state(h)) stride += (reg.second + 255) & ~size_t(255);
  int rc = h->alloc(&h->snap, stride * (size_t)slots);
  if (rc) return rc;
  h->snap_stride = stride;
  h->snap_slots = slots;
  h->snap_ok.assign((size_t)slots, 0);
  h->snap_fmt.assign((size_t)slots, 0);
  return 0;
} catch (...) {
  return host_error();
}

int sph_snapshot_save(SphHandle* h, int32_t slot, void* stream) try {
  if (!h || slot < 0 || slot >= h->snap_slots)
    return fail((int)SPH_ERR_INVALID_ARG, "snapshot slot out of range");
  if (!h->has_state || !steady(h))
    return fail((int)SPH_ERR_INVALID_ARG, "a snapshot is taken between two steps (after sph_step)");
  int rc = snap_copy(h, slot, true, (cudaStream_t)stream);
  if (!rc) {
    h->snap_ok[(size_t)slot] = 1;
    h->snap_fmt[(size_t)slot] = h->lean;
  }
  return rc;
} catch (...) {
  return host_error();
}

int sph_snapshot_restore(SphHandle* h, int32_t slot, void* stream) try {
  if (!h || slot < 0 || slot >= h->snap_slots || !h->snap_ok[(size_t)slot])
    return fail((int)SPH_ERR_INVALID_ARG, "no snapshot in that slot");
  if (h->snap_fmt[(size_t)slot] != h->lean)
    return fail((int)SPH_ERR_INVALID_ARG,
                "the snapshot's candidate lists are in another format than the passes now use");
  int rc = snap_copy(h, slot, false, (cudaStream_t)stream);
  if (rc) return rc;
  // the state between two steps: binned, lists built, a forward result and
  // bc_fn pending (what sph_snapshot_save required)
  h->has_state = h->binned = h->lists = h->from_forward = h->pending_bc = true;
  h->fresh = false;
  return 0;
} catch (...) {
  return host_error();
}

int sph_adjoint_init(SphHandle* h, int32_t slots) try {
  if (!h || slots <= 0) return fail((int)SPH_ERR_INVALID_ARG, "bad argument");
  const SphConfig& c = h->cfg;
  if (c.solver != SPH_SOLVER_SPH || c.is_rho_evol || c.is_heat_conduction || c.is_free_slip ||
      h->n_cases != 1)
    return fail((int)SPH_ERR_INVALID_ARG,
                "the adjoint covers one case of the SPH solver with density summation and, "
                "optionally, the no-slip generalized wall BC");
  const CaseDev& cd = h->hc[0];
  if (cd.av_alpha != 0.0f)
    return fail((int)SPH_ERR_INVALID_ARG, "the adjoint needs no artificial viscosity");
  if (c.is_bc_trick && (cd.g_kind != SPH_GEXT_ZERO || cd.bc_kind == SPH_BC_SOLID_ZERO_P ||
                        cd.bc_kind == SPH_BC_HT))
    return fail((int)SPH_ERR_INVALID_ARG,
                "the adjoint of the wall BC covers no external force and velocity-only bc_fn");
  if (h->tape_slots) return fail((int)SPH_ERR_INVALID_ARG, "adjoint tape already initialised");
  const long long N = h->N;
  const size_t S = (size_t)slots * N;
  int rc = h->alloc(&h->t_orig, S) | h->alloc(&h->t_meta, S) | h->alloc(&h->t_P4, S) |
           h->alloc(&h->t_U4, S) | h->alloc(&h->t_V4, S) | h->alloc(&h->t_R4, S) |
           h->alloc(&h->t_nbr, S * h->kmax) | h->alloc(&h->t_cnt, S) |
           h->alloc(&h->t_scr, 8 * (size_t)N) | h->alloc(&h->t_la, 3 * (size_t)N) |
           h->alloc(&h->t_lb, 3 * (size_t)N);
  if (rc) return rc;
  h->tape_slots = slots;
  return 0;
} catch (...) {
  return host_error();
}

int sph_tape_segment(SphHandle* h, int32_t nsteps, void* stream) try {
  if (!h || nsteps < 0 || nsteps > h->tape_slots)
    return fail((int)SPH_ERR_INVALID_ARG, "segment longer than the tape");
  for (int t = 0; t < nsteps; ++t) {
    int rc = sph_step(h, 1, stream);
    if (!rc) rc = sph_tape_record(h, t, stream);
    if (rc) return rc;
  }
  return 0;
} catch (...) {
  return host_error();
}

int sph_adjoint_segment(SphHandle* h, int32_t nsteps, float* lam_r, float* lam_u, float* lam_a,
                        float* lam_b, void* stream) try {
  if (!h || nsteps < 0 || nsteps > h->tape_slots)
    return fail((int)SPH_ERR_INVALID_ARG, "segment longer than the tape");
  for (int t = nsteps - 1; t >= 0; --t) {
    int rc = sph_adjoint_step(h, t, lam_r, lam_u, lam_a, lam_b, stream);
    if (rc) return rc;
  }
  return 0;
} catch (...) {
  return host_error();
}

int sph_tape_record(SphHandle* h, int32_t slot, void* stream) try {
  if (!h || slot < 0 || slot >= h->tape_slots)
    return fail((int)SPH_ERR_INVALID_ARG, "tape slot out of range");
  if (!(h->from_forward && h->pending_bc))
    return fail((int)SPH_ERR_INVALID_ARG, "record the tape right after sph_step");
  const long long N = h->N;
  const Buffers& b = h->buf[0];
  launch_tape_record(h->ctx((cudaStream_t)stream), b, h->R4, h->t_orig + slot * N,
                     h->t_P4 + slot * N, h->t_U4 + slot * N, h->t_V4 + slot * N,
                     h->t_R4 + slot * N, h->t_meta + slot * N,
                     h->t_nbr + (size_t)slot * h->kmax * N, h->t_cnt + slot * N);
  return launch_status("tape record");
} catch (...) {
  return host_error();
}

int sph_adjoint_step(SphHandle* h, int32_t slot, float* lam_r, float* lam_u, float* lam_a,
                     float* lam_b, void* stream) try {
  if (!h || slot < 0 || slot >= h->tape_slots)
    return fail((int)SPH_ERR_INVALID_ARG, "tape slot out of range");
  if (!lam_r || !lam_u || !lam_a || !lam_b)
    return fail((int)SPH_ERR_INVALID_ARG, "adjoint arrays missing");
  const long long N = h->N;
  cudaStream_t st = (cudaStream_t)stream;
  LaunchCtx L = h->ctx(st);
  AdjTape t{h->t_orig + slot * N, h->t_P4 + slot * N, h->t_U4 + slot * N,
            h->t_V4 + slot * N,   h->t_R4 + slot * N, h->t_meta + slot * N,
            h->t_nbr + (size_t)slot * h->kmax * N, h->t_cnt + slot * N};
  float4* p = h->t_scr;
  AdjScratch s{p, p + N, p + 2 * N, p + 3 * N, p + 4 * N, p + 5 * N, p + 6 * N, p + 7 * N};
  launch_adjoint(L, t, s, lam_a, lam_b, h->t_la, h->t_lb, lam_r, lam_u, h->cfg.is_bc_trick);
  const size_t bytes = sizeof(float) * (size_t)N * h->cfg.dim;
  cudaError_t e = cudaMemcpyAsync(lam_a, h->t_la, bytes, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(lam_b, h->t_lb, bytes, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return cuda_check(e, "adjoint copy");
  return launch_status("adjoint step");
} catch (...) {
  return host_error();
}

int sph_read_status(SphHandle* h, uint32_t* status, int32_t clear, void* stream) try {
  if (!h || !status) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, h->status, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && clear) e = cudaMemsetAsync(h->status, 0, sizeof(unsigned), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  int rc = cuda_check(e, "read status");
  *status = v;
  return rc;
} catch (...) {
  return host_error();
}

int sph_rebuild_stats(SphHandle* h, int64_t* rebuilds, int32_t* kernels_per_rebuild,
                      void* stream) try {
  if (!h || !rebuilds || !kernels_per_rebuild)
    return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, h->rebuilds_d, sizeof(v), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  *rebuilds = (int64_t)v + h->rebuilds_h;
  *kernels_per_rebuild = h->rebuild_launches;
  return cuda_check(e, "rebuild stats");
} catch (...) {
  return host_error();
}

int sph_read_status_async(SphHandle* h, uint32_t* status_dev, int32_t clear, void* stream) try {
  if (!h || !status_dev) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(status_dev, h->status, sizeof(unsigned),
                                  cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && clear) e = cudaMemsetAsync(h->status, 0, sizeof(unsigned), st);
  return cuda_check(e, "read status async");
} catch (...) {
  return host_error();
}

int sph_diagnostics(SphHandle* h, double* out, void* stream) try {
  if (!h || !out) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  launch_diagnostics(h->ctx((cudaStream_t)stream), h->buf[0], h->R4, h->from_forward,
                     h->pending_bc, out);
  return launch_status("diagnostics");
} catch (...) {
  return host_error();
}

int sph_neighbour_counts(SphHandle* h, int32_t* counts, void* stream) try {
  if (!h || !counts) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  if (!h->has_state || !h->from_forward || !h->binned)
    return fail((int)SPH_ERR_INVALID_ARG, "no forward pass since the state was loaded");
  launch_neighbour_counts(h->ctx((cudaStream_t)stream), h->buf[0], counts);
  return launch_status("neighbour counts");
} catch (...) {
  return host_error();
}

}  // extern "C"
