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
  Buffers buf[2]{};
  int cur = 0;
  float4* R4 = nullptr;
  float4* UT4 = nullptr;
  int* cellid = nullptr;
  int *count = nullptr, *start = nullptr, *keyc = nullptr, *keys = nullptr;
  int *tsrc = nullptr, *tkey = nullptr, *tcell = nullptr, *scan_tmp = nullptr;
  int *rowcnt = nullptr, *rowoff = nullptr;
  int *nbr = nullptr, *nbr_cnt = nullptr;
  int kmax = kListSlots;  // neighbour-list slots per particle
  int block = 256;        // threads per block of the forward passes
  unsigned* status = nullptr;
  unsigned long long* edgecnt = nullptr;
  const float* g_arr = nullptr;
  bool has_state = false, binned = false, from_forward = false, pending_bc = false;
  cudaStream_t hs = nullptr;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};  // one step from buffer parity 0 / 1
  const float* graph_g_arr = nullptr;
  int launch_count = 0;       // kernel launches of the last step
  cudaEvent_t* ev = nullptr;  // phase events while profiling
  // adjoint tape: per recorded step the sorted order, P4, U4, R4 and the
  // neighbour list of its forward pass
  int tape_slots = 0;
  int* t_orig = nullptr;
  float4 *t_P4 = nullptr, *t_U4 = nullptr, *t_R4 = nullptr;
  int *t_nbr = nullptr, *t_cnt = nullptr;
  float* t_mu = nullptr;
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
    L.block = block;
    L.launches = const_cast<int*>(&launch_count);
    L.ev = ev;
    return L;
  }
};

void sph::set_last_error(const std::string& msg) { g_last_error = msg; }

// Per-case float32 constants, rounded the way the reference's float32
// program rounds its Python-float parameters (weak types become float32).
int sph::make_case(const SphConfig& cfg, const SphCase& in, long long p_off, long long cell_off,
              CaseDev& c, std::string& err) {
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
  long long ncell = 1;
  for (int d = 0; d < 3; ++d) {
    c.nc[d] = nc[d];
    c.mult[d] = (int)ncell;
    ncell *= nc[d];
  }
  if (ncell > INT_MAX / 2) {
    err = "too many cells";
    return -1;
  }
  c.ncell = (int)ncell;
  c.cell_off = (int)cell_off;
  c.p_off = (int)p_off;
  c.n = (int)in.n;
  c.cell_cap = INT_MAX;
  c.edge_cap = LLONG_MAX;
  c.cutoff_sq = cut * cut;
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
  c.g_kind = in.g_kind;
  for (int d = 0; d < 3; ++d) {
    c.g[d] = (float)in.g[d];
    c.u_lid[d] = (float)in.u_lid[d];
  }
  c.g_lo = (float)in.g_band_lo;
  c.g_hi = (float)in.g_band_hi;
  c.bc_kind = in.bc_kind;
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
  if (c.fast) {
    c.cut_lo = (float)(c.cutoff_sq * (1.0 - rel));
    c.cut_hi = (float)(c.cutoff_sq * (1.0 + rel));
  } else {  // every candidate takes the reference metric
    c.cut_lo = -1.0f;
    c.cut_hi = INFINITY;
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
  for (int k = 0; k < 2; ++k) {
    if (h->gexec[k]) cudaGraphExecDestroy(h->gexec[k]);
    h->gexec[k] = nullptr;
  }
}

int launch_status(const char* what) { return cuda_check(cudaGetLastError(), what); }

// Re-bin the current positions without moving them; folds a pending forward
// result / bc_fn into the state buffers.
int bin_static(SphHandle* h, cudaStream_t st) {
  LaunchCtx L = h->ctx(st);
  Buffers in = h->buf[h->cur], out = h->buf[1 - h->cur];
  launch_bin(L, in, out, h->R4, h->cellid, h->count, h->start, h->keyc, h->keys, h->tsrc,
             h->tkey, h->tcell, h->scan_tmp, h->C, false, h->from_forward, h->pending_bc);
  h->cur = 1 - h->cur;
  h->binned = true;
  h->from_forward = false;
  h->pending_bc = false;
  return launch_status("bin");
}

// One si_euler step (integrator.py:22-56): kick-drift fused into the binning,
// forward pass, bc_fn (applied to accelerations in the force pass and folded
// into the state by the next binning / readback).
int step_once(SphHandle* h, cudaStream_t st) {
  h->launch_count = 0;
  LaunchCtx L = h->ctx(st);
  Buffers in = h->buf[h->cur], out = h->buf[1 - h->cur];
  launch_bin(L, in, out, h->R4, h->cellid, h->count, h->start, h->keyc, h->keys, h->tsrc,
             h->tkey, h->tcell, h->scan_tmp, h->C, true, h->from_forward, h->pending_bc);
  h->cur = 1 - h->cur;
  launch_forward(L, out, h->R4, h->R4, h->UT4, h->cellid, h->start, h->edgecnt, h->g_arr, true,
                 true);
  h->binned = true;
  h->from_forward = true;
  h->pending_bc = true;
  return launch_status("step");
}

bool steady(const SphHandle* h) { return h->from_forward && h->pending_bc; }

// Capture one step starting from the current buffer parity. Capture only
// records the launches; the host-side parity flip it performs is undone.
int capture_graph(SphHandle* h) {
  const int parity = h->cur;
  if (h->gexec[parity]) {
    cudaGraphExecDestroy(h->gexec[parity]);
    h->gexec[parity] = nullptr;
  }
  if (!h->hs) {
    cudaError_t e = cudaStreamCreateWithFlags(&h->hs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_check(e, "stream create");
  }
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(h->hs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_check(e, "begin capture");
  int rc = step_once(h, h->hs);
  e = cudaStreamEndCapture(h->hs, &graph);
  h->cur = parity;
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cuda_check(e, "end capture");
  e = cudaGraphInstantiate(&h->gexec[parity], graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_check(e, "graph instantiate");
  h->graph_g_arr = h->g_arr;
  return 0;
}

}  // namespace

extern "C" {

int sph_abi_version(void) { return SPH_ABI_VERSION; }

const char* sph_last_error(void) { return g_last_error.c_str(); }

int sph_create(const SphConfig* cfg, const SphCase* cases, int32_t n_cases, SphHandle** out) {
  if (!cfg || !cases || !out || n_cases <= 0)
    return fail((int)SPH_ERR_INVALID_ARG, "null argument or no cases");
  *out = nullptr;
  if (cfg->dim != 2 && cfg->dim != 3)
    return fail((int)SPH_ERR_INVALID_ARG, "Cell list spatial dimension must be 2 or 3");
  if (cfg->kernel != SPH_KERNEL_QSK && cfg->kernel != SPH_KERNEL_WC2K)
    return fail((int)SPH_ERR_INVALID_ARG, "kernel must be QSK or WC2K");
  if (cfg->solver != SPH_SOLVER_SPH && cfg->solver != SPH_SOLVER_RIE)
    return fail((int)SPH_ERR_INVALID_ARG, "solver must be SPH or RIE");
  if (n_cases >= (1 << 26)) return fail((int)SPH_ERR_INVALID_ARG, "too many cases");
  SphHandle* h = new SphHandle();
  h->cfg = *cfg;
  h->n_cases = n_cases;
  h->cases.assign(cases, cases + n_cases);
  h->hc.resize(n_cases);
  std::vector<long long> off(n_cases + 1, 0);
  long long cells = 0;
  for (int i = 0; i < n_cases; ++i) {
    if (cases[i].n <= 0) {
      delete h;
      return fail((int)SPH_ERR_INVALID_ARG, "every case needs at least one particle");
    }
    std::string err;
    if (make_case(*cfg, cases[i], off[i], cells, h->hc[i], err)) {
      delete h;
      return fail((int)SPH_ERR_INVALID_ARG, "case " + std::to_string(i) + ": " + err);
    }
    cells += h->hc[i].ncell;
    off[i + 1] = off[i] + cases[i].n;
  }
  h->N = off[n_cases];
  h->C = cells;
  if (h->N >= INT_MAX / 2 || h->C >= INT_MAX / 2) {
    delete h;
    return fail((int)SPH_ERR_INVALID_ARG, "problem too large for 32-bit indices");
  }
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
  }
  if (!rc) {
    rc |= h->alloc(&h->R4, N) | h->alloc(&h->cellid, N);
    if (cfg->solver == SPH_SOLVER_RIE) rc |= h->alloc(&h->UT4, N);
    rc |= h->alloc(&h->count, h->C + 1) | h->alloc(&h->start, h->C + 1) |
          h->alloc(&h->keyc, N) | h->alloc(&h->keys, N) | h->alloc(&h->tsrc, N) |
          h->alloc(&h->tkey, N) | h->alloc(&h->tcell, N) | h->alloc(&h->rowcnt, N + 1) |
          h->alloc(&h->rowoff, N + 1) | h->alloc(&h->nbr, (size_t)h->kmax * N) |
          h->alloc(&h->nbr_cnt, N);
    long long m = h->C + 1 > N + 1 ? h->C + 1 : N + 1;
    rc |= h->alloc(&h->scan_tmp, scan_tmp_ints(m));
    rc |= h->alloc(&h->status, 1) | h->alloc(&h->edgecnt, n_cases) | h->alloc(&h->dc, n_cases) |
          h->alloc(&h->case_off_d, n_cases + 1);
  }
  if (!rc) rc = cuda_check(cudaMemset(h->status, 0, sizeof(unsigned)), "memset");
  if (!rc)
    rc = cuda_check(cudaMemcpy(h->case_off_d, off.data(), sizeof(long long) * (n_cases + 1),
                               cudaMemcpyHostToDevice),
                    "upload offsets");
  if (!rc) rc = upload_cases(h, 0);
  if (rc) {
    for (void* p : h->allocs) cudaFree(p);
    delete h;
    return rc;
  }
  *out = h;
  return 0;
}

int sph_destroy(SphHandle* h) {
  if (!h) return 0;
  drop_graph(h);
  if (h->hs) cudaStreamDestroy(h->hs);
  for (void* p : h->allocs) cudaFree(p);
  delete h;
  return 0;
}

int sph_update_cases(SphHandle* h, const SphCase* cases, int32_t n_cases) {
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
  }
  h->cases.assign(cases, cases + n_cases);
  h->hc = next;
  drop_graph(h);
  return upload_cases(h, 0);
}

int sph_set_state(SphHandle* h, const SphStateView* s, void* stream) {
  if (!h || !s) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  if (s->n != h->N) return fail((int)SPH_ERR_INVALID_ARG, "state has the wrong particle count");
  if (!s->r || !s->tag || !s->u || !s->v || !s->dudt || !s->dvdt || !s->rho || !s->p ||
      !s->mass || !s->eta)
    return fail((int)SPH_ERR_INVALID_ARG, "missing state field");
  if (h->buf[0].NW4 && !s->nw)
    return fail((int)SPH_ERR_INVALID_ARG, "wall normals nw are required by this solver");
  bool garr = false;
  for (const auto& c : h->hc) garr |= c.g_kind == SPH_GEXT_ARRAY;
  if (garr && !s->g_ext)
    return fail((int)SPH_ERR_INVALID_ARG, "g_ext array required by SPH_GEXT_ARRAY");
  cudaStream_t st = (cudaStream_t)stream;
  h->cur = 0;
  launch_pack(h->ctx(st), *s, h->buf[0], h->case_off_d);
  h->g_arr = s->g_ext;
  h->has_state = true;
  h->binned = h->from_forward = h->pending_bc = false;
  return launch_status("set_state");
}

int sph_get_state(SphHandle* h, SphStateView* s, void* stream) {
  if (!h || !s) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  if (s->n != h->N) return fail((int)SPH_ERR_INVALID_ARG, "state has the wrong particle count");
  if (!s->r || !s->u || !s->v || !s->dudt || !s->dvdt || !s->rho || !s->p)
    return fail((int)SPH_ERR_INVALID_ARG, "missing state field");
  launch_unpack(h->ctx((cudaStream_t)stream), h->buf[h->cur], h->R4, *s, h->from_forward,
                h->pending_bc);
  return launch_status("get_state");
}

int sph_nl_update(SphHandle* h, void* stream) {
  if (!h) return fail((int)SPH_ERR_INVALID_ARG, "null handle");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  return bin_static(h, (cudaStream_t)stream);
}

int sph_nl_allocate(SphHandle* h, int64_t extra_capacity, SphNLCapacity* cap_out, void* stream) {
  if (!h) return fail((int)SPH_ERR_INVALID_ARG, "null handle");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  cudaStream_t st = (cudaStream_t)stream;
  // allocation sizes the capacities from the data and never flags an overflow
  for (auto& c : h->hc) {
    c.cell_cap = INT_MAX;
    c.edge_cap = LLONG_MAX;
  }
  int rc = upload_cases(h, st);
  if (!rc) rc = bin_static(h, st);
  if (rc) return rc;
  LaunchCtx L = h->ctx(st);
  launch_row_counts(L, h->buf[h->cur], h->cellid, h->start, h->rowcnt);
  if ((rc = launch_status("row counts"))) return rc;
  std::vector<int> start(h->C + 1), rows(h->N);
  cudaError_t e = cudaMemcpyAsync(start.data(), h->start, sizeof(int) * (h->C + 1),
                                  cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(rows.data(), h->rowcnt, sizeof(int) * h->N, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if ((rc = cuda_check(e, "allocate readback"))) return rc;
  const double mult = h->cfg.capacity_multiplier;
  const int nb = h->cfg.dim == 3 ? 27 : 9;
  for (int i = 0; i < h->n_cases; ++i) {
    CaseDev& c = h->hc[i];
    long long maxocc = 0, occ = 0;
    for (int k = 0; k < c.ncell; ++k) {
      long long o = start[c.cell_off + k + 1] - start[c.cell_off + k];
      maxocc = o > maxocc ? o : maxocc;
    }
    for (int k = 0; k < c.n; ++k) occ += rows[c.p_off + k];
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
  drop_graph(h);
  return upload_cases(h, st);
}

int sph_nl_set_capacity(SphHandle* h, const SphNLCapacity* cap) {
  if (!h || !cap) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  for (auto& c : h->hc) {
    c.cell_cap = (int)cap->cell_capacity;
    c.edge_cap = cap->max_occupancy;
  }
  drop_graph(h);
  return upload_cases(h, 0);
}

int sph_nl_edges(SphHandle* h, int32_t* idx, int64_t capacity, int64_t* count_dev,
                 void* stream) {
  if (!h || !idx || !count_dev || capacity < 0)
    return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  if (!h->binned) return fail((int)SPH_ERR_INVALID_ARG, "neighbour list not built");
  LaunchCtx L = h->ctx((cudaStream_t)stream);
  launch_edges(L, h->buf[h->cur], h->cellid, h->start, h->rowcnt, h->rowoff, h->scan_tmp, idx,
               capacity, (long long*)count_dev);
  return launch_status("edges");
}

int sph_forward(SphHandle* h, void* stream) {
  if (!h) return fail((int)SPH_ERR_INVALID_ARG, "null handle");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = 0;
  if (!h->binned || h->from_forward) rc = bin_static(h, st);
  if (rc) return rc;
  launch_forward(h->ctx(st), h->buf[h->cur], h->R4, h->R4, h->UT4, h->cellid, h->start,
                 h->edgecnt, h->g_arr, false, true);
  h->from_forward = true;
  h->pending_bc = false;
  return launch_status("forward");
}

int sph_step(SphHandle* h, int32_t nsteps, void* stream) {
  if (!h) return fail((int)SPH_ERR_INVALID_ARG, "null handle");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  if (nsteps < 0) return fail((int)SPH_ERR_INVALID_ARG, "negative step count");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = 0;
  // the first step after loading a state runs eagerly (it folds the loaded
  // state in); every later step replays the graph of its buffer parity
  if (nsteps > 0 && !steady(h)) {
    if ((rc = step_once(h, st))) return rc;
    --nsteps;
  }
  if (h->graph_g_arr != h->g_arr) drop_graph(h);
  while (nsteps > 0) {
    if (!h->gexec[h->cur] && (rc = capture_graph(h))) return rc;
    if ((rc = cuda_check(cudaGraphLaunch(h->gexec[h->cur], st), "graph launch"))) return rc;
    h->cur = 1 - h->cur;
    --nsteps;
  }
  return 0;
}

int sph_set_block_size(SphHandle* h, int32_t threads) {
  if (!h) return fail((int)SPH_ERR_INVALID_ARG, "null handle");
  if (threads < 32 || threads > 256 || threads % 32)
    return fail((int)SPH_ERR_INVALID_ARG, "block size must be a multiple of 32 in [32, 256]");
  h->block = threads;
  drop_graph(h);
  return 0;
}

int sph_step_launch_count(SphHandle* h, int32_t* count) {
  if (!h || !count) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  *count = h->launch_count;
  return 0;
}

int sph_profile_step(SphHandle* h, int32_t nsteps, float* ms, void* stream) {
  if (!h || !ms || nsteps <= 0) return fail((int)SPH_ERR_INVALID_ARG, "bad argument");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t ev[5];
  for (int k = 0; k < 5; ++k) cudaEventCreate(&ev[k]);
  for (int k = 0; k < 4; ++k) ms[k] = 0.f;
  int rc = 0;
  for (int i = 0; i < nsteps && !rc; ++i) {
    h->ev = ev;
    rc = step_once(h, st);
    h->ev = nullptr;
    if (rc) break;
    cudaError_t e = cudaEventSynchronize(ev[4]);
    if ((rc = cuda_check(e, "profile sync"))) break;
    for (int k = 0; k < 4; ++k) {
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
      ms[k] += t / nsteps;
    }
  }
  for (int k = 0; k < 5; ++k) cudaEventDestroy(ev[k]);
  return rc;
}

int sph_adjoint_init(SphHandle* h, int32_t slots) {
  if (!h || slots <= 0) return fail((int)SPH_ERR_INVALID_ARG, "bad argument");
  const SphConfig& c = h->cfg;
  if (c.solver != SPH_SOLVER_SPH || c.is_rho_evol || c.is_bc_trick || h->n_cases != 1)
    return fail((int)SPH_ERR_INVALID_ARG,
                "the adjoint covers one case of the SPH solver with density summation and "
                "no wall boundary condition");
  const CaseDev& cd = h->hc[0];
  if (cd.cv != 0.0f || cd.av_alpha != 0.0f)
    return fail((int)SPH_ERR_INVALID_ARG, "the adjoint needs tvf = 0 and no artificial viscosity");
  if (h->tape_slots) return fail((int)SPH_ERR_INVALID_ARG, "adjoint tape already initialised");
  const long long N = h->N;
  int rc = h->alloc(&h->t_orig, (size_t)slots * N) | h->alloc(&h->t_P4, (size_t)slots * N) |
           h->alloc(&h->t_U4, (size_t)slots * N) | h->alloc(&h->t_R4, (size_t)slots * N) |
           h->alloc(&h->t_nbr, (size_t)slots * h->kmax * N) |
           h->alloc(&h->t_cnt, (size_t)slots * N) | h->alloc(&h->t_mu, N);
  if (rc) return rc;
  h->tape_slots = slots;
  return 0;
}

int sph_tape_record(SphHandle* h, int32_t slot, void* stream) {
  if (!h || slot < 0 || slot >= h->tape_slots)
    return fail((int)SPH_ERR_INVALID_ARG, "tape slot out of range");
  if (!(h->from_forward && h->pending_bc))
    return fail((int)SPH_ERR_INVALID_ARG, "record the tape right after sph_step");
  cudaStream_t st = (cudaStream_t)stream;
  const long long N = h->N;
  const Buffers& b = h->buf[h->cur];
  cudaError_t e = cudaSuccess;
  auto cp = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st);
  };
  cp(h->t_orig + slot * N, b.ORIG, sizeof(int) * N);
  cp(h->t_P4 + slot * N, b.P4, sizeof(float4) * N);
  cp(h->t_U4 + slot * N, b.U4, sizeof(float4) * N);
  cp(h->t_R4 + slot * N, h->R4, sizeof(float4) * N);
  cp(h->t_nbr + (size_t)slot * h->kmax * N, h->nbr, sizeof(int) * h->kmax * N);
  cp(h->t_cnt + slot * N, h->nbr_cnt, sizeof(int) * N);
  return cuda_check(e, "tape record");
}

int sph_adjoint_step(SphHandle* h, int32_t slot, float* lam_r, float* lam_u,
                     const float* lam_a_in, float* lam_a_out, void* stream) {
  if (!h || slot < 0 || slot >= h->tape_slots)
    return fail((int)SPH_ERR_INVALID_ARG, "tape slot out of range");
  if (!lam_r || !lam_u || !lam_a_in || !lam_a_out || lam_a_in == lam_a_out)
    return fail((int)SPH_ERR_INVALID_ARG, "adjoint arrays missing or aliased");
  const long long N = h->N;
  LaunchCtx L = h->ctx((cudaStream_t)stream);
  launch_adjoint(L, h->t_orig + slot * N, h->t_P4 + slot * N, h->t_U4 + slot * N,
                 h->t_R4 + slot * N, h->t_nbr + (size_t)slot * h->kmax * N,
                 h->t_cnt + slot * N, h->t_mu, lam_a_in, lam_a_out, lam_r, lam_u);
  return launch_status("adjoint step");
}

int sph_read_status(SphHandle* h, uint32_t* status, int32_t clear, void* stream) {
  if (!h || !status) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, h->status, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && clear) e = cudaMemsetAsync(h->status, 0, sizeof(unsigned), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  int rc = cuda_check(e, "read status");
  *status = v;
  return rc;
}

int sph_diagnostics(SphHandle* h, double* out, void* stream) {
  if (!h || !out) return fail((int)SPH_ERR_INVALID_ARG, "null argument");
  if (!h->has_state) return fail((int)SPH_ERR_INVALID_ARG, "no state loaded");
  launch_diagnostics(h->ctx((cudaStream_t)stream), h->buf[h->cur], h->R4, h->from_forward,
                     h->pending_bc, out);
  return launch_status("diagnostics");
}

}  // extern "C"
