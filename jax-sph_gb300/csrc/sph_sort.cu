// Cell binning (counting sort by cell hash, stable by original index), state
// permutation with the fused si_euler kick-drift, exclusive scans, the sparse
// edge-list emitter and the float64 diagnostics.
//
// The sorted order equals the reference's `argsort(hashes)` (a stable sort of
// the original order, jax_md/partition.py:377): inside each cell particles are
// ranked by original index, so the result does not depend on atomic order.
#include "sph_internal.cuh"

namespace sph {

namespace {

constexpr int kBlock = 256;
constexpr unsigned kFull = 0xffffffffu;

inline int nblocks(long long n, int b = kBlock) { return (int)((n + b - 1) / b); }

__device__ __forceinline__ float4 ld4(const float* p, int dim, long long i) {
  float4 r;
  r.x = p[i * dim];
  r.y = p[i * dim + 1];
  r.z = dim == 3 ? p[i * dim + 2] : 0.0f;
  r.w = 0.0f;
  return r;
}
__device__ __forceinline__ void st3(float* p, int dim, long long i, float x, float y, float z) {
  if (!p) return;  // a field the caller does not read back
  p[i * dim] = x;
  p[i * dim + 1] = y;
  if (dim == 3) p[i * dim + 2] = z;
}

// ------------------------------------------------------------------ pack / unpack
// Load a state given in original order. With `inv` (the inverse permutation
// of the binning the buffers hold) every particle goes to its sorted slot, and
// `changed` is raised when a position differs (bitwise) from the one already
// there: the binning and candidate lists then still fit unless it is raised.
// A position that did not change keeps its float64 copy (precision form).
__global__ void k_pack(SphStateView s, int dim, Buffers o, const long long* case_off, int n_cases,
                       unsigned* status, const int* inv, unsigned* changed) {
  const long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  bool moved = false;
  if (i0 < s.n) {
    const long long i = i0;
    const long long q = inv ? inv[i] : i;
    int c = 0;
    while (c + 1 < n_cases && i >= case_off[c + 1]) ++c;
    int tag = s.tag[i];
    if (tag == SPH_TAG_PAD)
      tag = PAD;
    else if (tag < 0 || tag > 3)
      atomicOr(status, SPH_ERR_INVALID_ARG);
    float4 r = ld4(s.r, dim, i);
    r.w = s.mass[i];
    float4 u = ld4(s.u, dim, i);
    u.w = s.rho[i];
    // a drop-in step need not pass v: the kick recomputes it from u
    float4 v = s.v ? ld4(s.v, dim, i) : make_float4(0.f, 0.f, 0.f, 0.f);
    v.w = s.p ? s.p[i] : 0.0f;
    float4 a = ld4(s.dudt, dim, i);
    a.w = s.drhodt ? s.drhodt[i] : 0.0f;
    float4 b = ld4(s.dvdt, dim, i);
    if (inv) {
      const float4 old = o.P4[q];
      moved = __float_as_uint(old.x) != __float_as_uint(r.x) ||
              __float_as_uint(old.y) != __float_as_uint(r.y) ||
              (dim == 3 && __float_as_uint(old.z) != __float_as_uint(r.z));
    }
    o.P4[q] = r;
    o.U4[q] = u;
    o.V4[q] = v;
    o.A4[q] = a;
    o.A2[q] = b;
    o.ETA[q] = s.eta[i];
    o.META[q] = (c << kTagBits) | (tag & kTagMask);
    o.ORIG[q] = (int)i;
    if (o.NW4) o.NW4[q] = s.nw ? ld4(s.nw, dim, i) : make_float4(0.f, 0.f, 0.f, 0.f);
    if (o.TH4)
      o.TH4[q] = make_float4(s.T ? s.T[i] : 0.f, s.dTdt ? s.dTdt[i] : 0.f,
                             s.kappa ? s.kappa[i] : 0.f, s.Cp ? s.Cp[i] : 0.f);
    if (o.RD && (!inv || moved)) o.RD[q] = make_double4_32a(r.x, r.y, r.z, 0.0);
  }
  if (changed && __any_sync(0xffffffffu, moved) && (threadIdx.x & 31) == 0)
    atomicOr(changed, 1u);
}

// The state a step or forward left behind: density/pressure from the density
// pass (R4) when the buffers hold a forward result, bc_fn when a step ran.
struct Final {
  float3 u, v;
  float rho, p;
  float T, dTdt;  // heat conduction only
};
__device__ __forceinline__ Final finalize(const Buffers& b, const float4* R4, long long q,
                                          const CaseDev& c, int tag, bool from_forward,
                                          bool apply_bc) {
  float4 U = b.U4[q], V = b.V4[q];
  Final f;
  f.u = make_float3(U.x, U.y, U.z);
  f.v = make_float3(V.x, V.y, V.z);
  if (from_forward) {
    float4 R = R4[q];
    f.rho = R.x;
    f.p = R.y;
  } else {
    f.rho = U.w;
    f.p = V.w;
  }
  f.T = f.dTdt = 0.f;
  if (b.TH4) {
    if (from_forward) {
      const float2 t = b.TO[q];
      f.T = t.x;
      f.dTdt = t.y;
    } else {
      const float4 t = b.TH4[q];
      f.T = t.x;
      f.dTdt = t.y;
    }
  }
  if (apply_bc) {
    f.u = bc_vel(f.u, tag, c);
    f.v = bc_vel(f.v, tag, c);
    f.p = bc_p(f.p, tag, c);
    if (b.TH4) bc_temp(f.T, f.dTdt, tag, b.P4[q].x, c);
  }
  return f;
}

// Write the state back in the original order. With `ref` (device (n, dim)
// positions of a neighbour list) also the reference's rebuild test of that
// list (jax_md/partition.py:1010-1018): SPH_INFO_MOVED when some particle is
// farther than sqrt(thr_sq) from its reference position under the periodic
// metric.
__global__ void k_unpack(SphStateView s, int dim, Buffers b, const float4* R4,
                         const CaseDev* cases, bool from_forward, bool apply_bc,
                         const float* ref, float thr_sq, unsigned* status, const int* inv) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  bool moved = false;
  if (t < s.n) {
    // thread per original index (coalesced writes) when the inverse
    // permutation is known, else per sorted position
    const long long q = inv ? inv[t] : t;
    int meta = b.META[q];
    const CaseDev& c = cases[case_of(meta)];
    int tag = tag_of(meta);
    long long o = inv ? t : b.ORIG[q];
    Final f = finalize(b, R4, q, c, tag, from_forward, apply_bc);
    float4 r = b.P4[q], a = b.A4[q], a2 = b.A2[q];
    st3(s.r, dim, o, r.x, r.y, r.z);
    st3(s.u, dim, o, f.u.x, f.u.y, f.u.z);
    st3(s.v, dim, o, f.v.x, f.v.y, f.v.z);
    st3(s.dudt, dim, o, a.x, a.y, a.z);
    st3(s.dvdt, dim, o, a2.x, a2.y, a2.z);
    if (s.drhodt) s.drhodt[o] = a.w;
    if (s.rho) s.rho[o] = f.rho;
    if (s.p) s.p[o] = f.p;
    if (b.TH4) {
      if (s.T) s.T[o] = f.T;
      if (s.dTdt) s.dTdt[o] = f.dTdt;
    }
    if (s.nw && b.NW4) {  // the (possibly recomputed) wall normals
      const float4 n = b.NW4[q];
      st3(s.nw, dim, o, n.x, n.y, n.z);
    }
    if (ref) {
      const float4 r0 = make_float4(ref[o * dim], ref[o * dim + 1],
                                    dim == 3 ? ref[o * dim + 2] : 0.f, 0.f);
      float3 d;
      d.x = pdisp(__fsub_rn(r.x, r0.x), c.box[0], c.half[0]);
      d.y = pdisp(__fsub_rn(r.y, r0.y), c.box[1], c.half[1]);
      d.z = dim == 3 ? pdisp(__fsub_rn(r.z, r0.z), c.box[2], c.half[2]) : 0.f;
      const float d2 = dim == 3 ? sqd<3>(d) : sqd<2>(d);
      moved = d2 > thr_sq;
    }
  }
  if (__any_sync(0xffffffffu, moved) && (threadIdx.x & 31) == 0) atomicOr(status, SPH_INFO_MOVED);
}

// ------------------------------------------------------------------ binning
// si_euler kick-drift (integrator.py:26-30) in float32, one rounding per op.
template <int DIM>
__device__ __forceinline__ void kick_drift(float4& r, float3& u, float3& v, const float4& dudt,
                                           const float4& dvdt, const CaseDev& c) {
  u.x = __fadd_rn(u.x, __fmul_rn(c.dt, dudt.x));
  u.y = __fadd_rn(u.y, __fmul_rn(c.dt, dudt.y));
  v.x = __fadd_rn(u.x, __fmul_rn(c.cv, dvdt.x));
  v.y = __fadd_rn(u.y, __fmul_rn(c.cv, dvdt.y));
  r.x = jmod(__fadd_rn(r.x, __fmul_rn(c.dt, v.x)), c.box[0]);
  r.y = jmod(__fadd_rn(r.y, __fmul_rn(c.dt, v.y)), c.box[1]);
  if (DIM == 3) {
    u.z = __fadd_rn(u.z, __fmul_rn(c.dt, dudt.z));
    v.z = __fadd_rn(u.z, __fmul_rn(c.cv, dvdt.z));
    r.z = jmod(__fadd_rn(r.z, __fmul_rn(c.dt, v.z)), c.box[2]);
  }
}

// Precision form: the same kick in float32, the drift accumulated in float64
// (rd); the float32 position the passes read is rd rounded, kept below the
// box length.
__device__ __forceinline__ float drift_axis64(double& x, float v, double dt, double L, float Lf) {
  double y = x + dt * (double)v;
  if (y >= L) y -= L;
  else if (y < 0.0) y += L;
  x = y;
  const float f = (float)y;
  return f < Lf ? f : nextafterf(Lf, 0.f);
}

template <int DIM>
__device__ __forceinline__ void kick_drift64(float4& r, double4_32a& rd, float3& u, float3& v,
                                             const float4& dudt, const float4& dvdt,
                                             const CaseDev& c) {
  u.x = __fadd_rn(u.x, __fmul_rn(c.dt, dudt.x));
  u.y = __fadd_rn(u.y, __fmul_rn(c.dt, dudt.y));
  v.x = __fadd_rn(u.x, __fmul_rn(c.cv, dvdt.x));
  v.y = __fadd_rn(u.y, __fmul_rn(c.cv, dvdt.y));
  r.x = drift_axis64(rd.x, v.x, c.dt64, c.box64[0], c.box[0]);
  r.y = drift_axis64(rd.y, v.y, c.dt64, c.box64[1], c.box[1]);
  if (DIM == 3) {
    u.z = __fadd_rn(u.z, __fmul_rn(c.dt, dudt.z));
    v.z = __fadd_rn(u.z, __fmul_rn(c.cv, dvdt.z));
    r.z = drift_axis64(rd.z, v.z, c.dt64, c.box64[2], c.box[2]);
  }
}

// With `copy`, each thread first copies its particle's records from `src`
// into `in` (the scratch set the sort reads from): a rebuild's copy of the
// resident set rides along with the hashing instead of a copy per array.
template <int DIM>
__global__ void k_hash_count(long long N, Buffers in, const float4* R4, const CaseDev* cases,
                             int* count, int* keyc, int* keys, unsigned* status, bool drift,
                             bool from_forward, bool apply_bc, Buffers src, bool copy) {
  long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  bool valid = k < N;
  int cell = 0;
  if (valid && copy) {
    in.P4[k] = src.P4[k];
    in.U4[k] = src.U4[k];
    in.V4[k] = src.V4[k];
    in.A4[k] = src.A4[k];
    in.A2[k] = src.A2[k];
    in.ETA[k] = src.ETA[k];
    in.META[k] = src.META[k];
    in.ORIG[k] = src.ORIG[k];
    if (src.NW4) in.NW4[k] = src.NW4[k];
    if (src.RD) in.RD[k] = src.RD[k];
    if (src.TH4) in.TH4[k] = src.TH4[k];
  }
  if (valid) {
    int meta = in.META[k];
    const CaseDev& c = cases[case_of(meta)];
    float4 r = in.P4[k];
    if (drift) {
      Final f = finalize(in, R4, k, c, tag_of(meta), from_forward, apply_bc);
      float3 u = f.u, v;
      if (in.RD) {
        double4_32a rd = in.RD[k];
        kick_drift64<DIM>(r, rd, u, v, in.A4[k], in.A2[k], c);
      } else {
        kick_drift<DIM>(r, u, v, in.A4[k], in.A2[k], c);
      }
    }
    // padding goes to the parking cell past the grid: no walk visits it
    cell = c.cell_off + (tag_of(meta) == PAD ? c.ncell : cell_hash<DIM>(r, c, status));
  }
  unsigned mask = __ballot_sync(kFull, valid);
  if (!valid) return;
  // warp-aggregated slot reservation: lanes of one cell share one atomic
  unsigned peers = __match_any_sync(mask, cell);
  int lane = threadIdx.x & 31;
  int leader = __ffs(peers) - 1;
  int rank = __popc(peers & ((1u << lane) - 1u));
  int base = 0;
  if (lane == leader) base = atomicAdd(&count[cell], __popc(peers));
  base = __shfl_sync(peers, base, leader);
  keyc[k] = cell;
  keys[k] = base + rank;
}

__global__ void k_scatter(long long N, const int* keyc, const int* keys, const int* start,
                          const int* orig, int* tsrc, int* tkey, int* tcell) {
  long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k >= N) return;
  int cell = keyc[k];
  int q = start[cell] + keys[k];
  tsrc[q] = (int)k;
  tkey[q] = orig[k];
  tcell[q] = cell;
}

template <int DIM>
__global__ void k_permute(long long N, Buffers in, Buffers out, const float4* R4,
                          const CaseDev* cases, const int* start, const int* tsrc,
                          const int* tkey, const int* tcell, int* cellid, unsigned* status,
                          bool drift, bool from_forward, bool apply_bc, float4* rref,
                          int* inv) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  bool over = false;
  if (q < N) {
    int cell = tcell[q];
    int a = start[cell], e = start[cell + 1];
    int key = tkey[q];
    int rank = 0;
    for (int t = a; t < e; ++t) rank += (tkey[t] < key);
    int dest = a + rank;
    int src = tsrc[q];
    int meta = in.META[src];
    const CaseDev& c = cases[case_of(meta)];
    int tag = tag_of(meta);
    Final f = finalize(in, R4, src, c, tag, from_forward, apply_bc);
    float4 r = in.P4[src];
    float4 A = in.A4[src], B = in.A2[src];
    float3 u = f.u, v = f.v;
    if (in.RD) {
      double4_32a rd = in.RD[src];
      if (drift) kick_drift64<DIM>(r, rd, u, v, A, B, c);
      out.RD[dest] = rd;
    } else if (drift) {
      kick_drift<DIM>(r, u, v, A, B, c);
    }
    out.P4[dest] = r;
    out.U4[dest] = make_float4(u.x, u.y, u.z, f.rho);
    out.V4[dest] = make_float4(v.x, v.y, v.z, f.p);
    out.A4[dest] = A;
    out.A2[dest] = B;
    out.ETA[dest] = in.ETA[src];
    out.META[dest] = meta;
    out.ORIG[dest] = key;
    if (out.NW4) out.NW4[dest] = in.NW4[src];
    if (out.TH4) {
      const float4 t = in.TH4[src];
      out.TH4[dest] = make_float4(f.T, f.dTdt, t.z, t.w);
    }
    cellid[dest] = cell;
    if (rref) rref[dest] = r;
    if (inv) inv[key] = dest;
    // one test per occupied cell (of the grid), against the reference's cell
    if (c.use_cells && q == a && cell - c.cell_off < c.ncell)
      over = ref_cell_occupancy<DIM>(c, cell - c.cell_off, start) > c.cell_cap;
  }
  if (__any_sync(kFull, over) && (threadIdx.x & 31) == 0) atomicOr(status, SPH_CELL_LIST_OVERFLOW);
}

// One si_euler kick-drift (integrator.py:22-56) in place on the resident
// buffers, with the state folded in first (forward result, bc_fn). Two tests
// per particle ride along:
//  * the reference's cell-list capacity test of this step's update
//    (jax_md/partition.py:385-392): occupancy of the reference's cells,
//    counted with one atomic per cell present in a warp;
//  * the rebuild test: a rebuild of the candidate lists is due once the
//    minimum-image displacement since the last rebuild exceeds sqrt(v_dmax2).
template <int DIM>
__device__ __forceinline__ void kick_one(long long i, const Buffers& b, const float4* R4,
                                         const CaseDev& c, int meta, const float4* rref,
                                         unsigned* status, bool from_forward, bool apply_bc,
                                         bool& rebuild, int& key) {
  const Final f = finalize(b, R4, i, c, tag_of(meta), from_forward, apply_bc);
  float4 r = b.P4[i];
  float3 u = f.u, v;
  const float4 A = b.A4[i], B = b.A2[i];
  const float4 q = rref[i];
  if (b.RD) {
    double4_32a rd = b.RD[i];
    kick_drift64<DIM>(r, rd, u, v, A, B, c);
    b.RD[i] = rd;
  } else {
    kick_drift<DIM>(r, u, v, A, B, c);
  }
  b.P4[i] = r;
  b.U4[i] = make_float4(u.x, u.y, u.z, f.rho);
  b.V4[i] = make_float4(v.x, v.y, v.z, f.p);
  if (b.TH4) {
    const float4 t = b.TH4[i];
    b.TH4[i] = make_float4(f.T, f.dTdt, t.z, t.w);
  }
  float dx = r.x - q.x, dy = r.y - q.y, dz = (DIM == 3) ? r.z - q.z : 0.f;
  dx = fmaf(-c.box[0], rintf(dx * c.inv_box[0]), dx);
  dy = fmaf(-c.box[1], rintf(dy * c.inv_box[1]), dy);
  if (DIM == 3) dz = fmaf(-c.box[2], rintf(dz * c.inv_box[2]), dz);
  const bool pad = tag_of(meta) == PAD;  // no lists, no cell
  rebuild = !pad && !(dx * dx + dy * dy + dz * dz <= c.v_dmax2);  // NaN rebuilds too
  if (c.use_cells && !pad) {
    key = ref_cell_hash<DIM>(r, c);
    if (key < 0) atomicOr(status, SPH_ERR_NONFINITE);
    else key += c.cref_off;
  }
}

// ONE: a single case, its constants a kernel parameter (the capacity, which a
// capacity update changes without re-capturing the step, is read from the
// device copy).
template <int DIM, bool ONE>
__global__ void __launch_bounds__(kBlock, ONE ? 5 : 1)
k_kick(long long N, Buffers b, const float4* R4, const CaseDev c1, const CaseDev* cases,
       const float4* rref, int* cref_count, unsigned* vflag, unsigned* status,
       bool from_forward, bool apply_bc) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  bool rebuild = false, over = false;
  int key = -1, cap = 0;
  if (i < N) {
    const int meta = b.META[i];
    if (ONE) {
      kick_one<DIM>(i, b, R4, c1, meta, rref, status, from_forward, apply_bc, rebuild, key);
      if (key >= 0) cap = cases[0].cell_cap;
    } else {
      const CaseDev& c = cases[case_of(meta)];
      kick_one<DIM>(i, b, R4, c, meta, rref, status, from_forward, apply_bc, rebuild, key);
      cap = c.cell_cap;
    }
  }
  if (__any_sync(0xffffffffu, rebuild) && lane == 0) atomicOr(vflag, 1u);
  const unsigned m = __ballot_sync(0xffffffffu, key >= 0);
  if (key >= 0) {
    const unsigned peers = __match_any_sync(m, key);
    const int leader = __ffs(peers) - 1;
    if (lane == leader) {
      const int n = __popc(peers);
      over = atomicAdd(&cref_count[key], n) + n > cap;
    }
  }
  if (__any_sync(0xffffffffu, over) && lane == 0) atomicOr(status, SPH_CELL_LIST_OVERFLOW);
}

// Wall normals of the moved walls (a pass of its own so that the kick keeps
// its registers): walls point to their nearest layer point, fluid normals are 0.
template <int DIM>
__global__ void k_wall_normals(long long N, Buffers b, const CaseDev* cases, WallLayer layer) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int meta = b.META[i];
  b.NW4[i] = is_wall(tag_of(meta)) ? wall_normal<DIM>(b.P4[i], layer, cases[case_of(meta)])
                                   : make_float4(0.f, 0.f, 0.f, 0.f);
}

// ------------------------------------------------------------------ scan
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kTile = kScanThreads * kScanItems;

// Block-wide exclusive scan of kTile values; returns the tile total.
template <typename T>
__device__ T block_scan_tile(T* v /*[kScanItems]*/, T* smem /*[32]*/) {
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T local = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    T t = v[i];
    v[i] = local;
    local += t;
  }
  T x = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = smem[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(kFull, w, o);
      if (lane >= o) w += y;
    }
    smem[lane] = w;
  }
  __syncthreads();
  T warp_excl = warp > 0 ? smem[warp - 1] : 0;
  T total = smem[31];
  T excl = warp_excl + x - local;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) v[i] += excl;
  __syncthreads();
  return total;
}

// Per-tile totals of `n` values (summed in TO).
template <typename TI, typename TO>
__global__ void k_tile_sums(const TI* in, long long n, TO* sums) {
  __shared__ TO smem[32];
  long long base = blockIdx.x * (long long)kTile + threadIdx.x * kScanItems;
  TO v[kScanItems];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) v[i] = (base + i < n) ? (TO)in[base + i] : (TO)0;
  TO total = block_scan_tile(v, smem);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Exclusive scan of `n` values with an optional per-tile offset array;
// out[n] receives the grand total when this block owns the last tile.
template <typename TI, typename TO>
__global__ void k_tile_scan(const TI* in, long long n, TO* out, const TO* tile_off) {
  __shared__ TO smem[32];
  long long base = blockIdx.x * (long long)kTile + threadIdx.x * kScanItems;
  TO v[kScanItems];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) v[i] = (base + i < n) ? (TO)in[base + i] : (TO)0;
  TO total = block_scan_tile(v, smem);
  TO off = tile_off ? tile_off[blockIdx.x] : (TO)0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) out[base + i] = v[i] + off;
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = off + total;
}

// ------------------------------------------------------------------ edges
// The receivers c of sender s, i.e. the edges (c, s) with
// metric(r[s], r[c]) < cutoff_sq (jax_md/partition.py:885-909): the walk of
// the sender's cells (rows trimmed in fast cases) with the band test of the
// passes -- the shifted squared distance decides outside the band, the
// list's own rule inside it (every candidate without the fast test): the
// reference metric, or the matscipy backend's float64 distance.
template <int DIM, typename F>
__device__ __forceinline__ void for_each_receiver(const CaseDev& c, const CaseDev* cp, int cell,
                                                  const float4& rs, long long s, int mask_self,
                                                  const int* start, const float4* P4, F&& f) {
  auto visit = [&](int j0, int j1, float3 sh) {
    const float qx = rs.x - sh.x, qy = rs.y - sh.y, qz = rs.z - sh.z;
    for (int j = j0; j < j1; ++j) {
      if (mask_self && j == s) continue;
      const float4 rc = P4[j];
      bool e;
      if (c.fast) {
        const float dx = qx - rc.x, dy = qy - rc.y, dz = (DIM == 3) ? qz - rc.z : 0.f;
        const float d2 = dx * dx + dy * dy + dz * dz;
        // below the band an edge for either rule (the float64 cutoff^2 is
        // within 2^-24 of the float32 one, far inside the band)
        e = d2 < c.cut_lo || (d2 < c.cut_hi && list_edge<DIM>(rc, rs, cp));
      } else {
        e = list_edge<DIM>(rc, rs, cp);
      }
      if (e) f(j);
    }
  };
  if (c.fast)
    walk_rows<DIM, true>(c, cell, rs, start, c.rad, c.trim_r2, visit);
  else
    walk_rows<DIM, false>(c, cell, rs, start, c.rad, 0.f, visit);
}

// Per-sender edge count.
template <int DIM>
__global__ void k_row_counts(long long N, Buffers b, const CaseDev* cases, const int* cellid,
                             const int* start, int mask_self, int* rowcnt) {
  long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (s >= N) return;
  int meta = b.META[s];
  const CaseDev& c = cases[case_of(meta)];
  float4 rs = b.P4[s];
  int cnt = 0;
  if (tag_of(meta) == PAD) {  // padding is in no list
    rowcnt[b.ORIG[s]] = 0;
    return;
  }
  for_each_receiver<DIM>(c, cases + case_of(meta), cellid[s] - c.cell_off, rs, s, mask_self,
                         start, b.P4, [&](int) { ++cnt; });
  rowcnt[b.ORIG[s]] = cnt;
}

template <int DIM>
__global__ void k_emit(long long N, Buffers b, const CaseDev* cases, const int* cellid,
                       const int* start, int mask_self, const long long* rowoff, int32_t* idx,
                       long long capacity) {
  long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (s >= N) return;
  int meta = b.META[s];
  if (tag_of(meta) == PAD) return;
  const CaseDev& c = cases[case_of(meta)];
  float4 rs = b.P4[s];
  int sender = b.ORIG[s];
  long long off = rowoff[sender];
  long long k = off;
  for_each_receiver<DIM>(c, cases + case_of(meta), cellid[s] - c.cell_off, rs, s, mask_self,
                         start, b.P4, [&](int j) {
                           if (k < capacity) {
                             idx[k] = b.ORIG[j];
                             idx[capacity + k] = sender;
                           }
                           ++k;
                         });
  // receivers ascending per sender (insertion sort of the owned segment)
  long long end = k < capacity ? k : capacity;
  for (long long x = off + 1; x < end; ++x) {
    int key = idx[x];
    long long y = x - 1;
    while (y >= off && idx[y] > key) {
      idx[y + 1] = idx[y];
      --y;
    }
    idx[y + 1] = key;
  }
}

__global__ void k_pad_edges(int32_t* idx, long long capacity, const long long* total_ptr, int n,
                            long long* count_dev, unsigned* status) {
  long long total = *total_ptr;
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i == 0) {
    *count_dev = total;
    if (total > capacity) atomicOr(status, SPH_NEIGHBOR_LIST_OVERFLOW);
  }
  for (long long k = total + i; k < capacity; k += (long long)gridDim.x * blockDim.x) {
    idx[k] = n;
    idx[capacity + k] = n;
  }
}

// ------------------------------------------------------------------ diagnostics
__device__ __forceinline__ void atomic_max_pos(double* a, double v) {
  atomicMax((unsigned long long*)a, (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_min_pos(double* a, double v) {
  atomicMin((unsigned long long*)a, (unsigned long long)__double_as_longlong(v));
}

__global__ void k_diag_init(double* out, int n_cases) {
  int i = threadIdx.x + blockIdx.x * blockDim.x;
  if (i < n_cases * 8) {
    int k = i % 8;
    out[i] = k == 6 ? 1.0e300 : 0.0;
  }
}

template <int DIM>
__global__ void k_diagnostics(long long N, Buffers b, const float4* R4, const CaseDev* cases,
                              bool from_forward, bool apply_bc, double* out) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= N) return;
  int meta = b.META[q];
  int ci = case_of(meta);
  const CaseDev& c = cases[ci];
  int tag = tag_of(meta);
  Final f = finalize(b, R4, q, c, tag, from_forward, apply_bc);
  double* o = out + ci * 8;
  double umag = sqrt((double)f.u.x * f.u.x + (double)f.u.y * f.u.y + (double)f.u.z * f.u.z);
  atomic_max_pos(o + 5, umag);
  if (tag != FLUID) return;
  double m = b.P4[q].w;
  atomicAdd(o + 0, m);
  atomicAdd(o + 1, m * f.u.x);
  atomicAdd(o + 2, m * f.u.y);
  atomicAdd(o + 3, m * f.u.z);
  // get_ekin (jax_sph/utils.py:128-133): 0.5 * sum(v^2) * dx^dim over fluid
  double vol = DIM == 3 ? (double)c.av_hab * c.av_hab * c.av_hab : (double)c.av_hab * c.av_hab;
  atomicAdd(o + 4, 0.5 * vol *
                       ((double)f.v.x * f.v.x + (double)f.v.y * f.v.y + (double)f.v.z * f.v.z));
  atomic_min_pos(o + 6, (double)f.rho);
  atomic_max_pos(o + 7, (double)f.rho);
}

__global__ void k_neighbour_counts(long long N, const int* inv, const int* meta,
                                   const int* nbr_cnt, int self_term, int32_t* counts) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= N) return;
  const int q = inv[t];
  counts[t] = tag_of(meta[q]) == PAD ? 0 : (nbr_cnt[q] & ~kCountFlag) + self_term;
}

}  // namespace

// ------------------------------------------------------------------ launchers
// Scratch of a scan of n values, in ints: enough for 64-bit partial sums.
size_t scan_tmp_ints(long long n) { return 2 * ((size_t)((n + kTile - 1) / kTile) * 4 + 256); }

template <typename TI, typename TO>
int scan_t(cudaStream_t st, const TI* in, TO* out, long long n, TO* tmp) {
  long long tiles = (n + kTile - 1) / kTile;
  if (tiles <= 1) {
    k_tile_scan<TI, TO><<<1, kScanThreads, 0, st>>>(in, n, out, nullptr);
    return 1;
  }
  TO* sums = tmp;
  TO* offs = tmp + tiles + 1;
  k_tile_sums<TI, TO><<<(int)tiles, kScanThreads, 0, st>>>(in, n, sums);
  int k = scan_t<TO, TO>(st, sums, offs, tiles, tmp + 2 * tiles + 2);
  k_tile_scan<TI, TO><<<(int)tiles, kScanThreads, 0, st>>>(in, n, out, offs);
  return k + 2;
}

int launch_scan(cudaStream_t st, const int* in, int* out, long long n, int* tmp) {
  return scan_t<int, int>(st, in, out, n, tmp);
}

int launch_scan64(cudaStream_t st, const int* in, long long* out, long long n, int* tmp) {
  return scan_t<int, long long>(st, in, out, n, reinterpret_cast<long long*>(tmp));
}

void launch_pack(const LaunchCtx& L, const SphStateView& s, Buffers out,
                 const long long* case_off_dev, const int* inv, unsigned* changed) {
  k_pack<<<nblocks(L.N), kBlock, 0, L.stream>>>(s, L.dim, out, case_off_dev, L.n_cases, L.status,
                                                inv, changed);
  count_launch(L);
}

void launch_unpack(const LaunchCtx& L, Buffers in, const float4* R4, SphStateView& s,
                   bool from_forward, bool apply_bc, const float* ref, float thr_sq,
                   const int* inv) {
  k_unpack<<<nblocks(L.N), kBlock, 0, L.stream>>>(s, L.dim, in, R4, L.cases, from_forward,
                                                   apply_bc, ref, thr_sq, L.status, inv);
  count_launch(L);
}

void launch_bin(const LaunchCtx& L, Buffers in, Buffers out, const float4* R4, int* cellid,
                int* count, int* start, int* keyc, int* keys, int* tsrc, int* tkey, int* tcell,
                int* scan_tmp, long long total_cells, bool drift, bool from_forward,
                bool apply_bc, float4* rref, const Buffers* copy_src) {
  cudaMemsetAsync(count, 0, sizeof(int) * (total_cells + 1), L.stream);
  int g = nblocks(L.N);
  const Buffers src = copy_src ? *copy_src : in;
  if (L.dim == 3)
    k_hash_count<3><<<g, kBlock, 0, L.stream>>>(L.N, in, R4, L.cases, count, keyc, keys,
                                                 L.status, drift, from_forward, apply_bc, src,
                                                 copy_src != nullptr);
  else
    k_hash_count<2><<<g, kBlock, 0, L.stream>>>(L.N, in, R4, L.cases, count, keyc, keys,
                                                 L.status, drift, from_forward, apply_bc, src,
                                                 copy_src != nullptr);
  count_launch(L, 3 + launch_scan(L.stream, count, start, total_cells, scan_tmp));
  k_scatter<<<g, kBlock, 0, L.stream>>>(L.N, keyc, keys, start, in.ORIG, tsrc, tkey, tcell);
  if (L.dim == 3)
    k_permute<3><<<g, kBlock, 0, L.stream>>>(L.N, in, out, R4, L.cases, start, tsrc, tkey,
                                              tcell, cellid, L.status, drift, from_forward,
                                              apply_bc, rref, L.inv);
  else
    k_permute<2><<<g, kBlock, 0, L.stream>>>(L.N, in, out, R4, L.cases, start, tsrc, tkey,
                                              tcell, cellid, L.status, drift, from_forward,
                                              apply_bc, rref, L.inv);
}

void launch_kick(const LaunchCtx& L, Buffers b, const float4* R4, long long ref_cells,
                 bool from_forward, bool apply_bc) {
  if (ref_cells > 0) cudaMemsetAsync(L.cref_count, 0, sizeof(int) * ref_cells, L.stream);
  int g = nblocks(L.N);
#define SPH_KICK(D, ONE)                                                                      \
  k_kick<D, ONE><<<g, kBlock, 0, L.stream>>>(L.N, b, R4, L.c1, L.cases, L.rref, L.cref_count,  \
                                             L.vflag, L.status, from_forward, apply_bc)
  if (L.dim == 3) {
    if (L.n_cases == 1) SPH_KICK(3, true);
    else SPH_KICK(3, false);
  } else {
    if (L.n_cases == 1) SPH_KICK(2, true);
    else SPH_KICK(2, false);
  }
#undef SPH_KICK
  count_launch(L);
  // moving walls: the normals follow the new positions (integrator.py:33-34)
  if (L.layer.n > 0 && b.NW4) {
    if (L.dim == 3)
      k_wall_normals<3><<<g, kBlock, 0, L.stream>>>(L.N, b, L.cases, L.layer);
    else
      k_wall_normals<2><<<g, kBlock, 0, L.stream>>>(L.N, b, L.cases, L.layer);
    count_launch(L);
  }
}

// Capacities of an allocate (jax_md/partition.py:195-199, :956-971), per
// case: the largest occupancy of a reference cell (every occupied cell has a
// particle that sees it) and the number of edges (row counts, indexed by
// original particle). One atomic per case present in a warp.
__global__ void k_alloc_stats(long long N, Buffers b, const CaseDev* cases, const int* cellid,
                              const int* start, const int* rowcnt, int dim, int* case_max,
                              unsigned long long* case_edges) {
  const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const bool valid = s < N;
  int ci = 0, occ = 0, rows = 0;
  if (valid) {
    ci = case_of(b.META[s]);
    const CaseDev& c = cases[ci];
    const int cell = cellid[s] - c.cell_off;
    if (cell < c.ncell)  // padding sits in the parking cell, outside the grid
      occ = dim == 3 ? ref_cell_occupancy<3>(c, cell, start)
                     : ref_cell_occupancy<2>(c, cell, start);
    rows = rowcnt[b.ORIG[s]];
  }
  const unsigned mask = __ballot_sync(kFull, valid);
  if (!valid) return;
  const unsigned peers = __match_any_sync(mask, ci);
  const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
  const int m = __reduce_max_sync(peers, occ);
  const unsigned t = __reduce_add_sync(peers, (unsigned)rows);
  if (lane == leader) {
    atomicMax(&case_max[ci], m);
    atomicAdd(&case_edges[ci], (unsigned long long)t);
  }
}

void launch_alloc_stats(const LaunchCtx& L, Buffers b, const int* cellid, const int* start,
                        const int* rowcnt, int* case_max, unsigned long long* case_edges) {
  cudaMemsetAsync(case_max, 0, sizeof(int) * L.n_cases, L.stream);
  cudaMemsetAsync(case_edges, 0, sizeof(unsigned long long) * L.n_cases, L.stream);
  k_alloc_stats<<<nblocks(L.N), kBlock, 0, L.stream>>>(L.N, b, L.cases, cellid, start, rowcnt,
                                                       L.dim, case_max, case_edges);
}

void launch_row_counts(const LaunchCtx& L, Buffers b, const int* cellid, const int* start,
                       int* rowcnt) {
  int g = nblocks(L.N);
  if (L.dim == 3)
    k_row_counts<3><<<g, kBlock, 0, L.stream>>>(L.N, b, L.cases, cellid, start, L.mask_self,
                                                 rowcnt);
  else
    k_row_counts<2><<<g, kBlock, 0, L.stream>>>(L.N, b, L.cases, cellid, start, L.mask_self,
                                                 rowcnt);
}

void launch_edges(const LaunchCtx& L, Buffers b, const int* cellid, const int* start,
                  int* rowcnt, long long* rowoff, int* scan_tmp, int32_t* idx, long long capacity,
                  long long* count_dev) {
  launch_row_counts(L, b, cellid, start, rowcnt);
  // 64-bit edge offsets: the total can exceed 2^31 (dense clusters)
  launch_scan64(L.stream, rowcnt, rowoff, L.N, scan_tmp);
  int g = nblocks(L.N);
  if (L.dim == 3)
    k_emit<3><<<g, kBlock, 0, L.stream>>>(L.N, b, L.cases, cellid, start, L.mask_self, rowoff,
                                           idx, capacity);
  else
    k_emit<2><<<g, kBlock, 0, L.stream>>>(L.N, b, L.cases, cellid, start, L.mask_self, rowoff,
                                           idx, capacity);
  k_pad_edges<<<304, kBlock, 0, L.stream>>>(idx, capacity, rowoff + L.N, (int)L.N, count_dev,
                                            L.status);
}

void launch_neighbour_counts(const LaunchCtx& L, Buffers b, int32_t* counts) {
  k_neighbour_counts<<<nblocks(L.N), kBlock, 0, L.stream>>>(L.N, L.inv, b.META, L.nbr_cnt,
                                                            L.mask_self ? 0 : 1, counts);
}

void launch_diagnostics(const LaunchCtx& L, Buffers b, const float4* R4, bool from_forward,
                        bool apply_bc, double* out) {
  k_diag_init<<<nblocks(L.n_cases * 8), kBlock, 0, L.stream>>>(out, L.n_cases);
  int g = nblocks(L.N);
  if (L.dim == 3)
    k_diagnostics<3><<<g, kBlock, 0, L.stream>>>(L.N, b, R4, L.cases, from_forward, apply_bc,
                                                  out);
  else
    k_diagnostics<2><<<g, kBlock, 0, L.stream>>>(L.N, b, R4, L.cases, from_forward, apply_bc,
                                                  out);
}

}  // namespace sph
