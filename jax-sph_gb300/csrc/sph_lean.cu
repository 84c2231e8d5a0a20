// Lean candidate-list build, density pass and force pass for the plain
// drop-in configuration: one periodic case whose every axis has at least five
// reference cells (the fast membership test), standard SPH with density
// summation (solver.py:176-178, :794-796), standard + transport-velocity
// acceleration (:199-256), optional artificial viscosity (:404-428), no
// generalized wall BC, no heat conduction, pair sums in cell order. The
// neighbour sets, the membership test and the pair physics are those of the
// generic passes in sph_forward.cu; what differs is how the passes are fed:
//
//  * the case's constants arrive as a kernel parameter (constant bank), so
//    the hot loops take them as instruction operands instead of loading them
//    through a pointer into global memory;
//  * candidate and neighbour lists are k-major groups of four senders, one
//    load per group: either 16-bit offsets o = j - i of the sender's sorted
//    index from the receiver's, taken modulo the particle count, in an 8-byte
//    word (cells are sorted with the last axis slowest, so a neighbour across
//    that axis' periodic face is N minus a few planes away, i.e. a few planes
//    modulo N), or -- when a few planes of the case hold more than 16 bits
//    of particles -- 32-bit indices in a 16-byte word. A receiver with an
//    offset that does not fit, or with more candidates or neighbours than
//    slots, re-derives its senders from its cells instead;
//  * the candidate build walks, for every particle of a cell, the same cells
//    (those whose box lies within the list radius of the cell's box), so the
//    lanes of a warp stay converged;
//  * pair distances come from the reciprocal square root (at most 2 ulp)
//    rather than the correctly rounded square root, and the pair quotients
//    from the fast reciprocal; the float32 tolerances against the float64
//    oracle hold either way, and membership never depends on them (it is
//    decided on squared distances, exactly as in the generic passes).
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "sph_pairs.cuh"

namespace sph {

namespace {

constexpr unsigned kFull = 0xffffffffu;

inline int nblocks(long long n, int b) { return (int)((n + b - 1) / b); }

// ------------------------------------------------------------------ list formats
// A group of four list slots of one receiver. WIDE = false: four 16-bit
// offsets modulo n in a uint2; WIDE = true: four 32-bit indices in an int4.
template <bool WIDE>
struct Fmt;

template <>
struct Fmt<false> {
  using Word = uint2;
  // the slot's value for sender j (false: no 16-bit representative)
  static __device__ __forceinline__ bool enc(int i, int j, int n, int& o) {
    int d = j - i;
    if (d > 32767) d -= n;
    else if (d < -32768) d += n;
    o = d;
    return d >= -32768 && d <= 32767;
  }
  static __device__ __forceinline__ int raw(const Word& w, int q) {
    const unsigned h = (q & 2) ? w.y : w.x;
    return (int)(short)(unsigned short)(h >> ((q & 1) * 16));
  }
  // the sender of a slot's value
  static __device__ __forceinline__ int dec(int i, int o, int n) {
    int j = i + o;
    j += j < 0 ? n : 0;
    j -= j >= n ? n : 0;
    return j;
  }
  // the value that stands for the receiver itself (unused slots)
  static __device__ __forceinline__ int self(int) { return 0; }
  static __device__ __forceinline__ void put(Word* base, size_t stride, int k, int o) {
    reinterpret_cast<unsigned short*>(base + (size_t)(k >> 2) * stride)[k & 3] =
        (unsigned short)o;
  }
};

template <>
struct Fmt<true> {
  using Word = int4;
  static __device__ __forceinline__ bool enc(int, int j, int, int& o) {
    o = j;
    return true;
  }
  static __device__ __forceinline__ int raw(const Word& w, int q) {
    return q == 0 ? w.x : (q == 1 ? w.y : (q == 2 ? w.z : w.w));
  }
  static __device__ __forceinline__ int dec(int, int o, int) { return o; }
  static __device__ __forceinline__ int self(int i) { return i; }
  static __device__ __forceinline__ void put(Word* base, size_t stride, int k, int o) {
    reinterpret_cast<int*>(base + (size_t)(k >> 2) * stride)[k & 3] = o;
  }
};

// Minimum-image r_i - r_j and its square (the fast branch of pair_dr).
template <int DIM>
__device__ __forceinline__ void mi_dr(const float4& ri, const float4& rj, const CaseDev& c,
                                      float3& dr, float& d2) {
  dr.x = ri.x - rj.x;
  dr.y = ri.y - rj.y;
  dr.z = (DIM == 3) ? ri.z - rj.z : 0.f;
  dr.x = fmaf(-c.box[0], rintf(dr.x * c.inv_box[0]), dr.x);
  dr.y = fmaf(-c.box[1], rintf(dr.y * c.inv_box[1]), dr.y);
  if (DIM == 3) dr.z = fmaf(-c.box[2], rintf(dr.z * c.inv_box[2]), dr.z);
  d2 = dr.x * dr.x + dr.y * dr.y + dr.z * dr.z;
}

// Membership of (receiver ri, sender rj): below the band an edge, above it
// none, inside it the reference metric (jax_md/partition.py:897).
template <int DIM>
__device__ __forceinline__ bool lean_edge(const float4& ri, const float4& rj, const CaseDev& c,
                                          const CaseDev* cp, float3& dr, float& d2) {
  mi_dr<DIM>(ri, rj, c, dr, d2);
  bool in = d2 < c.cut_lo;
  if (!in && d2 < c.cut_hi) in = exact_edge<DIM>(ri, rj, cp);
  return in;
}

// |r| and 1/(|r| + eps) from r^2: 0 and 1/eps for coincident particles,
// like the reference's safe distance and its 1/(d + EPS).
__device__ __forceinline__ void dist_inv(float d2, float& dist, float& inv_d) {
  const float rs = rsqrtf(d2);
  dist = d2 > 0.f ? d2 * rs : 0.f;
  inv_d = d2 > 0.f ? rs : 1.0f / kEps;
}

// An upper bound of sqrt(x) for x > 0 (the reciprocal square root is within
// 2 ulp; the factor covers it).
__device__ __forceinline__ float sqrt_up(float x) { return x * rsqrtf(x) * 1.000001f; }

// Visit the candidates of a receiver at ri, binned into cell `cell`: the rows
// of cells whose box lies within sqrt(r2) of the cell's box (gaps between
// cell boxes, less the rounding margin; r* cells at most on each side) -- the
// same rows for every particle of a cell, so the lanes of a warp (receivers in
// neighbouring cells) run the row loop in step -- and in each row the cells
// within the chord of the particle's own sphere. A row is passed to f as one
// concatenated run of up to two contiguous ranges of the sorted order, the
// second where the row wraps around the periodic x face:
//   f(a0, n0, a1, n1, s1, sy, sz)   -- [a0, a0 + n0) unshifted in x,
//                                      [a1, a1 + n1) shifted by s1 in x,
// both shifted by (sy, sz) in y and z, so that one loop of n0 + n1 trips
// serves both and wrapping lanes do not diverge from the others.
template <int DIM, typename F>
__device__ __forceinline__ void box_rows(const CaseDev& c, int cell, const float4& ri,
                                         const int* __restrict__ start, int rx, int ry, int rz,
                                         float r2, F&& f) {
  const int nx = c.nc[0], ny = c.nc[1], nz = (DIM == 3) ? c.nc[2] : 1;
  const int cx = cell % nx;
  const int t = cell / nx;
  const int cy = t % ny;
  const int cz = (DIM == 3) ? t / ny : 0;
  const int* cs = start + c.cell_off;
  const float m = c.trim_m;
  const float R = sqrt_up(r2) + 2.f * m;
  const float R2 = R * R;
  const int zr = (DIM == 3) ? rz : 0;
  for (int dz = -zr; dz <= zr; ++dz) {
    const float gz = (float)max(abs(dz) - 1, 0) * c.cell_size[2];
    const float gz2 = (DIM == 3) ? gz * gz : 0.f;
    if (gz2 >= R2) continue;
    int zw = cz + dz;
    float sz = 0.f;
    if (zw < 0) { zw += nz; sz = -c.box[2]; }
    else if (zw >= nz) { zw -= nz; sz = c.box[2]; }
    // the particle's own gap to the plane (NaN for a non-finite position:
    // then no chord trimming below)
    float pz2 = 0.f;
    if (DIM == 3 && dz != 0) {
      const float g = (dz > 0 ? (float)(cz + dz) * c.cell_size[2] - ri.z
                              : ri.z - (float)(cz + dz + 1) * c.cell_size[2]) - m;
      pz2 = g > 0.f ? g * g : 0.f;
    }
    if (pz2 >= R2) continue;  // no row of this plane reaches the particle's sphere
    for (int dy = -ry; dy <= ry; ++dy) {
      const float gy = (float)max(abs(dy) - 1, 0) * c.cell_size[1];
      const float g2 = gz2 + gy * gy;
      if (g2 >= R2) continue;
      // the particle's own gap to the row: a row its sphere does not reach
      // holds no candidate and is skipped before any of its bookkeeping
      float p2 = pz2;
      if (dy != 0) {
        const float g = (dy > 0 ? (float)(cy + dy) * c.cell_size[1] - ri.y
                                : ri.y - (float)(cy + dy + 1) * c.cell_size[1]) - m;
        p2 += g > 0.f ? g * g : 0.f;
      }
      if (p2 >= R2) continue;
      int yw = cy + dy;
      float sy = 0.f;
      if (yw < 0) { yw += ny; sy = -c.box[1]; }
      else if (yw >= ny) { yw -= ny; sy = c.box[1]; }
      const int kx = min(rx, 1 + (int)(sqrt_up(R2 - g2) * c.inv_cs[0]));
      int xa = cx - kx, xb = cx + kx;
      {
        // the chord of the particle's sphere through this row
        const float w = sqrt_up(R2 - p2) + m;
        const float lo = floorf((ri.x - w) * c.inv_cs[0]);
        const float hi = floorf((ri.x + w) * c.inv_cs[0]);
        const int ta = (int)fminf(fmaxf(lo, (float)xa), (float)xb);
        const int tb = (int)fminf(fmaxf(hi, (float)xa), (float)xb);
        xa = ta;
        xb = tb;
      }
      const int row = (zw * ny + yw) * nx;
      int a0, e0, a1 = 0, e1 = 0;
      float s1 = 0.f;
      if (xb < xa) {
        a0 = e0 = 0;
      } else if (xa < 0) {
        a0 = cs[row];
        e0 = cs[row + xb + 1];
        a1 = cs[row + xa + nx];
        e1 = cs[row + nx];
        s1 = -c.box[0];
      } else if (xb >= nx) {
        a0 = cs[row + xa];
        e0 = cs[row + nx];
        a1 = cs[row];
        e1 = cs[row + xb - nx + 1];
        s1 = c.box[0];
      } else {
        a0 = cs[row + xa];
        e0 = cs[row + xb + 1];
      }
      f(a0, e0 - a0, a1, e1 - a1, s1, sy, sz);
    }
  }
}

// Senders j != i that are edges of receiver i, the slow way: its candidate
// list when every candidate fitted (but the neighbours did not), else the
// walk of the cells around its cell at the last binning, where every sender
// now within the cutoff was within the list radius.
template <int DIM, bool WIDE, typename F>
__device__ __forceinline__ void lean_slow(int N, int i, const float4& ri, const CaseDev& c,
                                          const CaseDev* cp, const float4* __restrict__ P4,
                                          const typename Fmt<WIDE>::Word* vl, const int* vcnt,
                                          int kv, const int* cellid, const int* start,
                                          const float4* rref, F&& f) {
  using L = Fmt<WIDE>;
  auto test = [&](int j) {
    const float4 rj = __ldg(P4 + j);
    float3 dr;
    float d2;
    if (lean_edge<DIM>(ri, rj, c, cp, dr, d2)) f(j, rj, dr, d2);
  };
  const int vc = vcnt[i];
  if (vc <= kv) {
    for (int k = 0; k < vc; ++k) test(L::dec(i, L::raw(vl[(size_t)(k >> 2) * N + i], k & 3), N));
    return;
  }
  box_rows<DIM>(c, cellid[i] - c.cell_off, rref[i], start, c.vrad[0], c.vrad[1], c.vrad[2],
                c.v_r2, [&](int a0, int n0, int a1, int n1, float, float, float) {
                  for (int t = 0; t < n0 + n1; ++t) {
                    const int j = t < n0 ? a0 + t : a1 + (t - n0);
                    if (j != i) test(j);
                  }
                });
}

// ------------------------------------------------------------------ candidates
// The senders within the list radius of every receiver at the current
// binning (shifted squared distance < v_r2), self excluded, in walk (cell)
// order. The loop over a range is branch-free: every candidate's slot value
// is stored at the next free slot of the receiver's column in shared memory
// and the count advances only for a member; the column is then copied to the
// k-major list in whole words. vcnt = kv + 1 marks a receiver whose
// candidates do not all fit (too many, or an offset beyond 16 bits): the
// passes walk its cells instead.
template <int DIM, bool WIDE>
__global__ void __launch_bounds__(256)
k_verlet_lean(int N, Buffers b, const CaseDev c, const int* __restrict__ cellid,
              const int* __restrict__ start, typename Fmt<WIDE>::Word* vl, int* vcnt, int kv) {
  using L = Fmt<WIDE>;
  extern __shared__ __align__(16) unsigned char s_raw[];  // [kv][blockDim.x] sender indices
  const int bs = blockDim.x;
  int* col = reinterpret_cast<int*>(s_raw) + threadIdx.x;
  const int i = blockIdx.x * bs + threadIdx.x;
  if (i >= N) return;
  if (tag_of(b.META[i]) == PAD) {
    vcnt[i] = 0;
    return;
  }
  const float4 ri = b.P4[i];
  const float r2 = c.v_r2;
  int m = 0;
  box_rows<DIM>(c, cellid[i] - c.cell_off, ri, start, c.vrad[0], c.vrad[1], c.vrad[2], r2,
                [&](int a0, int n0, int a1, int n1, float s1, float sy, float sz) {
    const float qx0 = ri.x, qx1 = ri.x - s1, qy = ri.y - sy, qz = ri.z - sz;
    const int d1 = a1 - n0;
    const int n = n0 + n1;
#pragma unroll 2
    for (int t = 0; t < n; ++t) {
      const bool second = t >= n0;
      const int j = t + (second ? d1 : a0);
      const float4 rj = __ldg(b.P4 + j);
      const float dx = (second ? qx1 : qx0) - rj.x, dy = qy - rj.y;
      const float dz = (DIM == 3) ? qz - rj.z : 0.f;
      const bool in = j != i && dx * dx + dy * dy + dz * dz < r2;
      col[(m < kv ? m : kv - 1) * bs] = j;
      m += in;
    }
  });
  bool wide = false;
  if (m <= kv) {
    typename L::Word* out = vl + i;
    for (int k = 0; k < m; ++k) {
      int o;
      wide |= !L::enc(i, col[k * bs], N, o);
      L::put(out, (size_t)N, k, o);
    }
  }
  vcnt[i] = (wide || m > kv) ? kv + 1 : m;
}

// Edge count for the NEIGHBOR_LIST_OVERFLOW test (one case). The capacity is
// read from the device copy of the case: a capacity update does not
// re-capture the step's graph.
__device__ __forceinline__ void count_edges1(int cnt, bool valid, unsigned long long* edgecnt,
                                             const CaseDev* cp, unsigned* status) {
  const unsigned mask = __ballot_sync(kFull, valid);
  if (!valid) return;
  const unsigned tot = __reduce_add_sync(mask, (unsigned)cnt);
  if ((threadIdx.x & 31) == __ffs(mask) - 1) {
    const unsigned long long old = atomicAdd(edgecnt, (unsigned long long)tot);
    if ((long long)(old + tot) > cp->edge_cap) atomicOr(status, SPH_NEIGHBOR_LIST_OVERFLOW);
  }
}

// ------------------------------------------------------------------ density
// The density filter of a receiver whose candidates did not fit its list
// (the case from its device copy).
template <int DIM, int KER, bool KAHAN, bool WIDE>
struct DensitySlow {
  Acc<KAHAN> s;
  int m, wide;
};
template <int DIM, int KER, bool KAHAN, bool WIDE>
__device__ __forceinline__ DensitySlow<DIM, KER, KAHAN, WIDE> density_slow(
    int N, int i, float4 ri, bool fluid, Acc<KAHAN> s0, const CaseDev* cp, const float4* P4,
    const typename Fmt<WIDE>::Word* vl, const int* vcnt, int kv, const int* cellid,
    const int* start, const float4* rref, typename Fmt<WIDE>::Word* srow, int bs, int kmax) {
  using L = Fmt<WIDE>;
  const CaseDev& c = *cp;
  int m = 0;
  bool wide = false;
  lean_slow<DIM, WIDE>(N, i, ri, c, cp, P4, vl, vcnt, kv, cellid, start, rref,
                       [&](int j, const float4&, const float3&, float d2) {
                         if (fluid) {
                           float dist, inv_d;
                           dist_inv(d2, dist, inv_d);
                           s0.add(kw<KER>(dist, c));
                         }
                         int o;
                         wide |= !L::enc(i, j, N, o);
                         if (m < kmax) L::put(srow, (size_t)bs, m, o);
                         ++m;
                       });
  return {s0, m, wide ? 1 : 0};
}

// Summation density (rho_i = m_i sum_j W_ij over the edges, self pair
// included unless masked; fluid receivers), Tait / Riemann EOS, and the
// step's neighbour list (staged in shared memory, written k-major) for the
// force pass. Candidates are filtered four at a time: one list word, four
// independent position gathers. R4 = (rho, p, V^2 = (m / rho)^2, eta): the
// force pass takes the volumes from there.
template <int DIM, int KER, bool KAHAN, bool WIDE>
__global__ void __launch_bounds__(256, 4)
k_density_lean(int N, Buffers b, const CaseDev c, const CaseDev* cp, int self_term,
               const int* __restrict__ cellid, const int* __restrict__ start,
               const typename Fmt<WIDE>::Word* __restrict__ vl, const int* __restrict__ vcnt,
               int kv, typename Fmt<WIDE>::Word* nb, int* nbcnt, int kmax, float4* R4,
               const float4* __restrict__ rref, unsigned long long* edgecnt, unsigned* status) {
  using L = Fmt<WIDE>;
  using Word = typename L::Word;
  extern __shared__ __align__(16) unsigned char s_raw[];  // [kmax / 4][blockDim.x] words
  Word* s_nb = reinterpret_cast<Word*>(s_raw);
  const int tid = threadIdx.x, bs = blockDim.x;
  const int i = blockIdx.x * bs + tid;
  const bool valid = i < N;
  int cnt = 0;
  if (valid) {
    const int tag = tag_of(b.META[i]);
    const bool fluid = tag == FLUID;
    const float4 ri = b.P4[i];
    Acc<KAHAN> s0;
    if (fluid && self_term) s0.add(kw<KER>(0.f, c));
    Word* srow = s_nb + tid;
    int m = 0;
    bool wide = false;
    const int vc = vcnt[i];
    if (vc <= kv) {
      const Word* vli = vl + i;
      const int ng = (vc + 3) >> 2;
      unsigned long long band = 0;  // list slots of candidates in the band
      Word wn = vli[0];  // (read even without candidates: never used then)
      for (int g = 0; g < ng; ++g) {
        const Word w = wn;
        if (g + 1 < ng) wn = vli[(size_t)(g + 1) * N];
        const int rem = vc - 4 * g;
        int o[4];
        float4 rj[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          // slots past the count hold stale words: they stand for i itself
          o[q] = q < rem ? L::raw(w, q) : L::self(i);
          rj[q] = __ldg(b.P4 + L::dec(i, o[q], N));
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float3 dr;
          float d2;
          mi_dr<DIM>(ri, rj[q], c, dr, d2);
          const bool e = q < rem && d2 < c.cut_lo;
          // a candidate in the band around the cutoff is decided after the
          // loop: few receivers have one, but nearly every group of a warp
          // would otherwise run the reference metric for some lane
          const int k = 4 * g + q;
          if (q < rem && !e && d2 < c.cut_hi && k < 64) band |= 1ull << k;
          if (e) {
            if (fluid) {
              float dist, inv_d;
              dist_inv(d2, dist, inv_d);
              s0.add(kw<KER>(dist, c));
            }
            if (m < kmax) L::put(srow, (size_t)bs, m, o[q]);
            ++m;
          }
        }
      }
      // the band's candidates in list order (slots beyond the mask's 64
      // re-tested): the reference metric decides (jax_md/partition.py:897),
      // and an edge joins the list after the others
      for (int k = 0; k < vc; ++k) {
        if (k < 64) {
          if (!band) {
            k = 63;  // no more masked slots
            continue;
          }
          k = __ffsll((long long)band) - 1;
          band &= band - 1;
        }
        const int o = L::raw(vli[(size_t)(k >> 2) * N], k & 3);
        const float4 rj = __ldg(b.P4 + L::dec(i, o, N));
        float3 dr;
        float d2;
        mi_dr<DIM>(ri, rj, c, dr, d2);
        if (k >= 64 && !(!(d2 < c.cut_lo) && d2 < c.cut_hi)) continue;
        if (exact_edge<DIM>(ri, rj, cp)) {
          if (fluid) {
            float dist, inv_d;
            dist_inv(d2, dist, inv_d);
            s0.add(kw<KER>(dist, c));
          }
          if (m < kmax) L::put(srow, (size_t)bs, m, o);
          ++m;
        }
      }
    } else {
      const DensitySlow<DIM, KER, KAHAN, WIDE> r = density_slow<DIM, KER, KAHAN, WIDE>(
          N, i, ri, fluid, s0, cp, b.P4, vl, vcnt, kv, cellid, start, rref, srow, bs, kmax);
      s0 = r.s;
      m = r.m;
      wide = r.wide != 0;
    }
    cnt = tag == PAD ? 0 : m + (self_term ? 1 : 0);
    // a receiver whose senders do not fit the format keeps its count, flagged
    nbcnt[i] = wide ? (m | kCountFlag) : m;
    if (!wide && m <= kmax) {
      const int ng = (m + 3) >> 2;
      for (int g = 0; g < ng; ++g) nb[(size_t)g * N + i] = s_nb[g * bs + tid];
    }
    const float rho_i = b.U4[i].w;
    const float rho_new = fluid ? ri.w * s0.s : rho_i;
    const float p_new = eos_p(rho_new, c);
    const float V = ri.w / rho_new;
    R4[i] = make_float4(rho_new, p_new, V * V, b.ETA[i]);
    if (!isfinite(rho_new) || !isfinite(p_new)) atomicOr(status, SPH_ERR_NONFINITE);
  }
  count_edges1(cnt, valid, edgecnt, cp, status);
}

// ------------------------------------------------------------------ force
// The receiver's own quantities of the force pass.
struct ForceI {
  float4 ri;
  float3 ui, hAi, wi;  // hAi = rho_i u_i / 2
  float rho_i, p_i, eta_i, Vi2, inv_mi;
  bool fluid;
};

template <bool KAHAN>
struct Acc6 {
  Acc<KAHAN> ax, ay, az, tx, ty, tz;
};

// One pair of the standard acceleration with the transport-velocity stress
// (solver.py:216-256), the transport-velocity acceleration (:199-213) and the
// artificial viscosity (:404-428, decided at compile time). The volumes
// squared, V^2 = (m / rho)^2, come from the density pass (R4.z).
template <int DIM, int KER, bool KAHAN, bool AV>
__device__ __forceinline__ void force_pair(const ForceI& I, const CaseDev& c, const int* meta,
                                             int j, const float4& rj, const float4& Uj4,
                                             const float4& Vj4, const float4& Rj,
                                             const float3& dr, float d2, Acc6<KAHAN>& A) {
  float dist, inv_d;
  dist_inv(d2, dist, inv_d);
  const float gw = kdw<KER>(dist, c);
  const float rho_j = Rj.x, p_j = Rj.y, eta_j = Rj.w;
  const float cc = (I.Vi2 + Rj.z) * I.inv_mi * gw * inv_d;
  const float3 uj = f3(Uj4);
  const float3 vj = f3(Vj4);
  const float eta_ij = __fdividef(2.f * I.eta_i * eta_j, I.eta_i + eta_j + kEps);
  const float p_ij = __fdividef(rho_j * I.p_i + I.rho_i * p_j, I.rho_i + rho_j);
  const float ki = dot3(I.wi, dr);
  const float kj = dot3(make_float3(vj.x - uj.x, vj.y - uj.y, vj.z - uj.z), dr);
  // the stress term (A_i ki + rho_j u_j kj) / 2 as (A_i / 2) ki + (rho_j kj / 2) u_j:
  // the halvings are exact, rho_j kj / 2 is formed once per pair
  const float hk = 0.5f * rho_j * kj;
  const float3 du = make_float3(I.ui.x - uj.x, I.ui.y - uj.y, I.ui.z - uj.z);
  float3 a = make_float3(cc * (fmaf(-p_ij, dr.x, fmaf(I.hAi.x, ki, hk * uj.x)) + eta_ij * du.x),
                         cc * (fmaf(-p_ij, dr.y, fmaf(I.hAi.y, ki, hk * uj.y)) + eta_ij * du.y),
                         cc * (fmaf(-p_ij, dr.z, fmaf(I.hAi.z, ki, hk * uj.z)) + eta_ij * du.z));
  if (AV && I.fluid && tag_of(meta[j]) == FLUID) {
    const float m_j = rj.w;
    const float rho_ab = 0.5f * (I.rho_i + rho_j);
    const float num = m_j * c.av_alpha * c.av_hab * c.av_cab *
                      (du.x * dr.x + du.y * dr.y + du.z * dr.z);
    const float k = num * gw * inv_d / (rho_ab * (dist * dist + c.av_eps));
    a.x += k * dr.x;
    a.y += k * dr.y;
    a.z += k * dr.z;
  }
  A.ax.add(a.x);
  A.ay.add(a.y);
  A.az.add(a.z);
  const float ct = cc * c.p_bg_tvf;
  A.tx.add(ct * dr.x);
  A.ty.add(ct * dr.y);
  A.tz.add(ct * dr.z);
}

// The force sums of a receiver whose neighbours did not fit its list (the
// case from its device copy).
template <int DIM, int KER, bool KAHAN, bool WIDE, bool AV>
__device__ __forceinline__ Acc6<KAHAN> force_slow(int N, int i, ForceI I, Acc6<KAHAN> A,
                                                 const CaseDev* cp, Buffers b,
                                                 const float4* R4,
                                                 const typename Fmt<WIDE>::Word* vl,
                                                 const int* vcnt, int kv, const int* cellid,
                                                 const int* start, const float4* rref) {
  const CaseDev& c = *cp;
  lean_slow<DIM, WIDE>(N, i, I.ri, c, cp, b.P4, vl, vcnt, kv, cellid, start, rref,
                       [&](int j, const float4& rj, const float3& dr, float d2) {
                         force_pair<DIM, KER, KAHAN, AV>(I, c, b.META, j, rj,
                                                           __ldg(b.U4 + j), __ldg(b.V4 + j),
                                                           __ldg(R4 + j), dr, d2, A);
                       });
  return A;
}

// The force pass over the density pass's neighbour list and its
// R4 = (rho, p, V^2, eta), with g_ext and bc_fn; the next sender's four
// records are in flight while a pair is evaluated, and the list word after
// the current one a group ahead. drho/dt is the receiver's own (a summation
// density carries it over).
template <int DIM, int KER, bool KAHAN, bool WIDE, bool AV>
__global__ void __launch_bounds__(256, 3)
k_force_lean(int N, Buffers b, const CaseDev c, const CaseDev* cp, const float* g_arr,
               const float4* __restrict__ R4, const typename Fmt<WIDE>::Word* __restrict__ nb,
               const int* __restrict__ nbcnt, int kmax, const typename Fmt<WIDE>::Word* vl,
               const int* vcnt, int kv, const int* cellid, const int* start, const float4* rref,
               bool apply_bc, unsigned* status) {
  using L = Fmt<WIDE>;
  using Word = typename L::Word;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int tag = tag_of(b.META[i]);
  ForceI I;
  I.ri = b.P4[i];
  I.fluid = tag == FLUID;
  I.ui = f3(b.U4[i]);
  const float3 vi = f3(b.V4[i]);
  const float4 Ri = R4[i];
  const float drhodt = b.A4[i].w;
  I.rho_i = Ri.x;
  I.p_i = Ri.y;
  I.eta_i = Ri.w;
  I.Vi2 = Ri.z;
  I.inv_mi = 1.0f / I.ri.w;
  I.hAi = make_float3(0.5f * (I.rho_i * I.ui.x), 0.5f * (I.rho_i * I.ui.y),
                      0.5f * (I.rho_i * I.ui.z));
  I.wi = make_float3(vi.x - I.ui.x, vi.y - I.ui.y, vi.z - I.ui.z);
  const float3 gi = g_ext<DIM>(c, I.ri, g_arr, c.g_kind == SPH_GEXT_ARRAY ? b.ORIG[i] : 0);
  Acc6<KAHAN> A;
  const int m = nbcnt[i];
  if (m <= kmax) {
    const Word* nbi = nb + i;
    const int ng = (m + 3) >> 2;
    Word wn = nbi[0];  // (read even without neighbours: never used then)
    int jn = m > 0 ? L::dec(i, L::raw(wn, 0), N) : i;
    float4 rn = __ldg(b.P4 + jn), un = __ldg(b.U4 + jn), vn = __ldg(b.V4 + jn),
           Rn = __ldg(R4 + jn);
    for (int g = 0; g < ng; ++g) {
      const Word w = wn;
      if (g + 1 < ng) wn = nbi[(size_t)(g + 1) * N];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int k = 4 * g + q;
        if (k < m) {
          const int jc = jn;
          const float4 rc = rn, uc = un, vc = vn, Rc = Rn;
          const int on = q < 3 ? L::raw(w, q + 1) : L::raw(wn, 0);
          jn = k + 1 < m ? L::dec(i, on, N) : i;
          rn = __ldg(b.P4 + jn);
          un = __ldg(b.U4 + jn);
          vn = __ldg(b.V4 + jn);
          Rn = __ldg(R4 + jn);
          float3 dr;
          float d2;
          mi_dr<DIM>(I.ri, rc, c, dr, d2);
          force_pair<DIM, KER, KAHAN, AV>(I, c, b.META, jc, rc, uc, vc, Rc, dr, d2, A);
        }
      }
    }
  } else {
    A = force_slow<DIM, KER, KAHAN, WIDE, AV>(N, i, I, A, cp, b, R4, vl, vcnt, kv, cellid,
                                                start, rref);
  }
  float3 dudt = make_float3(A.ax.s + gi.x, A.ay.s + gi.y, A.az.s + gi.z);
  float3 dvdt = make_float3(A.tx.s, A.ty.s, A.tz.s);
  if (DIM == 2) {
    dudt.z = 0.f;
    dvdt.z = 0.f;
  }
  if (apply_bc) {
    dudt = bc_acc(dudt, tag, c);
    dvdt = bc_acc(dvdt, tag, c);
  }
  if (!isfinite(dudt.x) || !isfinite(dudt.y) || !isfinite(dudt.z))
    atomicOr(status, SPH_ERR_NONFINITE);
  b.A4[i] = make_float4(dudt.x, dudt.y, dudt.z, drhodt);
  b.A2[i] = make_float4(dvdt.x, dvdt.y, dvdt.z, 0.f);
}

// ------------------------------------------------------------------ staged force
// The force pass with its senders staged in shared memory, one plane of
// cells at a time (the tiled form of the pass). A block's receivers are
// consecutive in the sorted order; when they share one plane of the binning,
// the senders of their lists lie in the planes dz = -rz..rz around it, and in
// each plane in the rows within the list radius of the receivers' rows --
// one or two contiguous ranges of the sorted order (two where the rows wrap
// around the periodic y face). Stage s copies plane s's ranges (four records
// per sender: r + m, u, v, R4) into shared memory with 1-D bulk copies, one
// per range and record array, whose bytes complete an mbarrier phase (a copy
// that does not complete within the poll limit sets SPH_ERR_TIMEOUT and the
// pass reads every sender from global memory instead); every receiver then walks
// its list from where it stopped, taking a sender from shared memory while it
// lies in the staged ranges and stopping at the first one that lies in a
// later stage's. A sender in no staged range (a list entry of the cutoff band,
// appended after the walk order; rows beyond the tile's capacity) is read from
// global memory in place. Each receiver thus evaluates its pairs in list order
// with the same arithmetic as k_force_lean: the results are the same bits.
// Blocks whose receivers span two planes stage nothing.
constexpr int kMaxStages = 9;

struct StageWin {
  int a0, n0, a1, n1;
};

// The ranges of the stage at plane offset dz for receivers in rows ya..yb of
// plane cz, truncated to `cap` senders.
template <int DIM>
__device__ __forceinline__ StageWin stage_window(const CaseDev& c, const int* cs, int cz, int ya,
                                                 int yb, int dz, int cap) {
  StageWin w{0, 0, 0, 0};
  const int nx = c.nc[0], ny = c.nc[1], nz = (DIM == 3) ? c.nc[2] : 1;
  // rows whose cell boxes lie within the list radius of the receivers' rows
  // (the gaps box_rows skips on; larger by the rounding margin)
  const float R = sqrt_up(c.v_r2) + 2.f * c.trim_m;
  const float gz = (float)max(abs(dz) - 1, 0) * c.cell_size[2];
  const float rem = R * R - ((DIM == 3) ? gz * gz : 0.f);
  if (rem <= 0.f) return w;
  const int ky = min(c.vrad[1], 1 + (int)(sqrt_up(rem) * (1.0f / c.cell_size[1])));
  int zw = cz + dz;
  zw += zw < 0 ? nz : 0;
  zw -= zw >= nz ? nz : 0;
  const int base = zw * ny;
  const int yl = ya - ky, yh = yb + ky;
  if (yh - yl + 1 >= ny) {
    w.a0 = cs[base * nx];
    w.n0 = cs[(base + ny) * nx] - w.a0;
  } else if (yl < 0) {
    w.a0 = cs[(base + yl + ny) * nx];
    w.n0 = cs[(base + ny) * nx] - w.a0;
    w.a1 = cs[base * nx];
    w.n1 = cs[(base + yh + 1) * nx] - w.a1;
  } else if (yh >= ny) {
    w.a0 = cs[(base + yl) * nx];
    w.n0 = cs[(base + ny) * nx] - w.a0;
    w.a1 = cs[base * nx];
    w.n1 = cs[(base + yh - ny + 1) * nx] - w.a1;
  } else {
    w.a0 = cs[(base + yl) * nx];
    w.n0 = cs[(base + yh + 1) * nx] - w.a0;
  }
  w.n0 = min(w.n0, cap);
  w.n1 = min(w.n1, cap - w.n0);
  return w;
}

// 1-D bulk copies (cp.async.bulk) of global ranges into shared memory, their
// completion counted in bytes on an mbarrier; every wait is bounded.
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// orders this thread's earlier shared-memory accesses before later
// async-proxy (bulk copy) writes
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// dst and src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_to_smem(void* dst, const void* src, unsigned bytes,
                                             unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// polls phase `parity` of the barrier at most `polls` times (false: gave up)
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int polls) {
  for (int it = 0; it < polls; ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
constexpr int kStagePolls = 1 << 20;

__device__ __forceinline__ int win_slot(const StageWin& w, int j) {
  if ((unsigned)(j - w.a0) < (unsigned)w.n0) return j - w.a0;
  if ((unsigned)(j - w.a1) < (unsigned)w.n1) return w.n0 + (j - w.a1);
  return -1;
}

template <int DIM, int KER, bool KAHAN, bool WIDE, bool AV>
__global__ void __launch_bounds__(128, 5)
k_force_staged(int N, Buffers b, const CaseDev c, const CaseDev* cp, const float* g_arr,
               const float4* __restrict__ R4, const typename Fmt<WIDE>::Word* __restrict__ nb,
               const int* __restrict__ nbcnt, int kmax, const typename Fmt<WIDE>::Word* vl,
               const int* vcnt, int kv, const int* cellid, const int* start, const float4* rref,
               bool apply_bc, unsigned* status, int cap) {
  using L = Fmt<WIDE>;
  using Word = typename L::Word;
  extern __shared__ __align__(16) float4 s_rec[];  // [4][cap]: r + m, u, v, R4
  __shared__ StageWin s_win[kMaxStages];
  __shared__ int s_ns;
  __shared__ __align__(8) unsigned long long s_bar;  // completion of a stage's copies
  if (threadIdx.x == 0) mbar_init(&s_bar, 1);
  const int i0 = blockIdx.x * blockDim.x;
  const int i = i0 + threadIdx.x;
  const bool live = i < N;
  if (threadIdx.x < kMaxStages) {
    // every thread of the first warp finds the block's plane; thread s
    // computes stage s
    const int* cs = start + c.cell_off;
    const int nx = c.nc[0], ny = c.nc[1], nz = (DIM == 3) ? c.nc[2] : 1;
    const int i1 = min(i0 + (int)blockDim.x, N) - 1;
    const int ca = cellid[i0] - c.cell_off, cb = cellid[i1] - c.cell_off;
    const int za = ca / (nx * ny), zb = cb / (nx * ny);
    const int rz = (DIM == 3) ? c.vrad[2] : 0;
    const int ns = 2 * rz + 1;
    // one plane per block, no plane visited twice, within the stage table
    const bool ok = za == zb && ns <= kMaxStages && ns <= nz;
    const int s = threadIdx.x;
    if (ok && s < ns)
      s_win[s] = stage_window<DIM>(c, cs, za, (ca / nx) % ny, (cb / nx) % ny, s - rz, cap);
    if (s == 0) s_ns = ok ? ns : 0;
  }
  ForceI I;
  int tag = PAD, m = 0;
  float drhodt = 0.f;
  float3 gi = make_float3(0.f, 0.f, 0.f);
  if (live) {
    tag = tag_of(b.META[i]);
    I.ri = b.P4[i];
    I.fluid = tag == FLUID;
    I.ui = f3(b.U4[i]);
    const float3 vi = f3(b.V4[i]);
    const float4 Ri = R4[i];
    drhodt = b.A4[i].w;
    I.rho_i = Ri.x;
    I.p_i = Ri.y;
    I.eta_i = Ri.w;
    I.Vi2 = Ri.z;
    I.inv_mi = 1.0f / I.ri.w;
    I.hAi = make_float3(0.5f * (I.rho_i * I.ui.x), 0.5f * (I.rho_i * I.ui.y),
                        0.5f * (I.rho_i * I.ui.z));
    I.wi = make_float3(vi.x - I.ui.x, vi.y - I.ui.y, vi.z - I.ui.z);
    gi = g_ext<DIM>(c, I.ri, g_arr, c.g_kind == SPH_GEXT_ARRAY ? b.ORIG[i] : 0);
    m = nbcnt[i];
  }
  const bool listed = live && m <= kmax;
  Acc6<KAHAN> A;
  const Word* nbi = nb + (live ? i : 0);
  int k = 0, wg = -1;
  Word w{};
  __syncthreads();
  const int ns = s_ns;
  int nstage = ns;  // stages staged in shared memory (0 once a copy timed out)
  unsigned phase = 0u;
  // stages 0..ns-1, then a last pass without a staged range for what is left
  // (one evaluation site for every listed pair)
  for (int s = 0; s <= ns; ++s) {
    StageWin cur{0, 0, 0, 0};
    if (s < nstage) {  // uniform over the block
      if (s > 0) {
        fence_proxy_async_smem();
        __syncthreads();  // the previous stage's reads are done
      }
      cur = s_win[s];
      const int nw = cur.n0 + cur.n1;
      if (nw > 0) {
        // the stage's ranges of the four record arrays: one bulk copy each
        if (threadIdx.x == 0) {
          mbar_expect_tx(&s_bar, 64u * (unsigned)nw);
          const float4* src[4] = {b.P4, b.U4, b.V4, R4};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            if (cur.n0 > 0)
              bulk_to_smem(s_rec + q * cap, src[q] + cur.a0, 16u * (unsigned)cur.n0, &s_bar);
            if (cur.n1 > 0)
              bulk_to_smem(s_rec + q * cap + cur.n0, src[q] + cur.a1, 16u * (unsigned)cur.n1,
                           &s_bar);
          }
        }
        const bool ok = mbar_wait(&s_bar, phase, kStagePolls);
        if (__syncthreads_or(!ok)) {
          // a copy that did not complete: report it, wait (bounded) for what
          // is in flight, and read every sender from global memory instead
          if (threadIdx.x == 0) atomicOr(status, SPH_ERR_TIMEOUT);
          mbar_wait(&s_bar, phase, kStagePolls);
          nstage = 0;
          cur = StageWin{0, 0, 0, 0};
        }
        phase ^= 1u;
      }
    }
    if (!listed) continue;
    while (k < m) {
      if ((k >> 2) != wg) {
        wg = k >> 2;
        w = nbi[(size_t)wg * N];
      }
      const int j = L::dec(i, L::raw(w, k & 3), N);
      const int t = win_slot(cur, j);
      float4 rj, uj, vj, Rj;
      if (t >= 0) {
        rj = s_rec[t];
        uj = s_rec[cap + t];
        vj = s_rec[2 * cap + t];
        Rj = s_rec[3 * cap + t];
      } else {
        bool later = false;
        for (int s2 = s + 1; s2 < nstage; ++s2) later |= win_slot(s_win[s2], j) >= 0;
        if (later) break;
        rj = __ldg(b.P4 + j);
        uj = __ldg(b.U4 + j);
        vj = __ldg(b.V4 + j);
        Rj = __ldg(R4 + j);
      }
      float3 dr;
      float d2;
      mi_dr<DIM>(I.ri, rj, c, dr, d2);
      force_pair<DIM, KER, KAHAN, AV>(I, c, b.META, j, rj, uj, vj, Rj, dr, d2, A);
      ++k;
    }
  }
  if (!live) return;
  if (!listed) {
    A = force_slow<DIM, KER, KAHAN, WIDE, AV>(N, i, I, A, cp, b, R4, vl, vcnt, kv, cellid,
                                                start, rref);
  }
  float3 dudt = make_float3(A.ax.s + gi.x, A.ay.s + gi.y, A.az.s + gi.z);
  float3 dvdt = make_float3(A.tx.s, A.ty.s, A.tz.s);
  if (DIM == 2) {
    dudt.z = 0.f;
    dvdt.z = 0.f;
  }
  if (apply_bc) {
    dudt = bc_acc(dudt, tag, c);
    dvdt = bc_acc(dvdt, tag, c);
  }
  if (!isfinite(dudt.x) || !isfinite(dudt.y) || !isfinite(dudt.z))
    atomicOr(status, SPH_ERR_NONFINITE);
  b.A4[i] = make_float4(dudt.x, dudt.y, dudt.z, drhodt);
  b.A2[i] = make_float4(dvdt.x, dvdt.y, dvdt.z, 0.f);
}

// Senders staged per stage: the rows a block of `bt` receivers spans at the
// case's mean row occupancy, plus the list radius' rows on each side, with a
// tenth in reserve (a stage holding more reads the rest from global memory).
inline int staged_capacity(const CaseDev& c, int dim, int bt) {
  const double rows = (double)c.nc[1] * (dim == 3 ? (double)c.nc[2] : 1.0);
  const double per_row = (double)c.n / rows;
  const double spanned = std::ceil(bt / std::max(per_row, 1.0)) + 1.0;
  const double win = (spanned + 2.0 * c.vrad[1]) * per_row * 1.1;
  // at most 46 KB per block: with the static stage table within the 48 KB a
  // launch may take without opting in
  const int cap = (int)std::min(win, 46.0 * 1024 / 64);
  return std::max(32, std::min((cap + 31) / 32 * 32, 736));
}

template <int DIM, int KER, bool KAHAN, bool WIDE>
void forward_lean_t(const LaunchCtx& L, Buffers b, float4* R4, const int* cellid,
                    const int* start, unsigned long long* edgecnt, const float* g_arr,
                    bool apply_bc, int phases) {
  using Word = typename Fmt<WIDE>::Word;
  const int bt = L.block > 0 ? L.block : 256;
  const int g = nblocks(L.N, bt);
  const int N = (int)L.N;
  Word* vl = reinterpret_cast<Word*>(L.vl);
  Word* nb = reinterpret_cast<Word*>(L.nbr);
  if (phases & 1) {
    const size_t smem = sizeof(Word) * (L.kmax / 4) * bt;
    k_density_lean<DIM, KER, KAHAN, WIDE><<<g, bt, smem, L.stream>>>(
        N, b, L.c1, L.cases, !L.mask_self, cellid, start, vl, L.vcnt, L.kv, nb, L.nbr_cnt,
        L.kmax, R4, L.rref, edgecnt, L.status);
    count_launch(L);
    mark(L, 2);
    mark(L, 3);
  }
  if ((phases & 2) && L.force_variant == SPH_FORCE_STAGED) {
    const int sb = 128;
    const int cap = staged_capacity(L.c1, L.dim, sb);
    const size_t smem = sizeof(float4) * 4 * (size_t)cap;
    if (L.c1.av_alpha != 0.0f)
      k_force_staged<DIM, KER, KAHAN, WIDE, true><<<nblocks(N, sb), sb, smem, L.stream>>>(
          N, b, L.c1, L.cases, g_arr, R4, nb, L.nbr_cnt, L.kmax, vl, L.vcnt, L.kv, cellid,
          start, L.rref, apply_bc, L.status, cap);
    else
      k_force_staged<DIM, KER, KAHAN, WIDE, false><<<nblocks(N, sb), sb, smem, L.stream>>>(
          N, b, L.c1, L.cases, g_arr, R4, nb, L.nbr_cnt, L.kmax, vl, L.vcnt, L.kv, cellid,
          start, L.rref, apply_bc, L.status, cap);
    count_launch(L);
    mark(L, 4);
  } else if (phases & 2) {
    if (L.c1.av_alpha != 0.0f)
      k_force_lean<DIM, KER, KAHAN, WIDE, true><<<g, bt, 0, L.stream>>>(
          N, b, L.c1, L.cases, g_arr, R4, nb, L.nbr_cnt, L.kmax, vl, L.vcnt, L.kv, cellid,
          start, L.rref, apply_bc, L.status);
    else
      k_force_lean<DIM, KER, KAHAN, WIDE, false><<<g, bt, 0, L.stream>>>(
          N, b, L.c1, L.cases, g_arr, R4, nb, L.nbr_cnt, L.kmax, vl, L.vcnt, L.kv, cellid,
          start, L.rref, apply_bc, L.status);
    count_launch(L);
    mark(L, 4);
  }
}

template <int DIM, int KER, bool KAHAN>
void forward_lean_w(const LaunchCtx& L, Buffers b, float4* R4, const int* cellid,
                    const int* start, unsigned long long* edgecnt, const float* g_arr,
                    bool apply_bc, int phases) {
  if (L.lean == 2)
    forward_lean_t<DIM, KER, KAHAN, true>(L, b, R4, cellid, start, edgecnt, g_arr, apply_bc,
                                          phases);
  else
    forward_lean_t<DIM, KER, KAHAN, false>(L, b, R4, cellid, start, edgecnt, g_arr, apply_bc,
                                           phases);
}

template <int DIM, int KER>
void forward_lean_k(const LaunchCtx& L, Buffers b, float4* R4, const int* cellid,
                    const int* start, unsigned long long* edgecnt, const float* g_arr,
                    bool apply_bc, int phases) {
  if (L.kahan)
    forward_lean_w<DIM, KER, true>(L, b, R4, cellid, start, edgecnt, g_arr, apply_bc, phases);
  else
    forward_lean_w<DIM, KER, false>(L, b, R4, cellid, start, edgecnt, g_arr, apply_bc, phases);
}

template <int DIM, bool WIDE>
void verlet_lean_t(const LaunchCtx& L, Buffers b, const int* cellid, const int* start) {
  using Word = typename Fmt<WIDE>::Word;
  // the staging column of kv sender indices per thread stays within 48 KB
  const int col = 4 * L.kv;
  int bt = (49152 / col) / 32 * 32;
  bt = bt > 256 ? 256 : bt;
  const size_t smem = (size_t)col * bt;
  k_verlet_lean<DIM, WIDE><<<nblocks(L.N, bt), bt, smem, L.stream>>>(
      (int)L.N, b, L.c1, cellid, start, reinterpret_cast<Word*>(L.vl), L.vcnt, L.kv);
}

}  // namespace

int lean_config(const SphConfig& cfg, int n_cases, const CaseDev& c0) {
  if (!(n_cases == 1 && c0.fast && cfg.solver == SPH_SOLVER_SPH && !cfg.is_rho_evol &&
        !cfg.is_heat_conduction && !cfg.canonical_order && !cfg.is_bc_trick &&
        cfg.nl_backend == SPH_NL_JAXMD && c0.n < (1 << 30)))
    return 0;
  // 16-bit offsets when a sender lies at most vrad + 1 cells away along the
  // slowest axis (the sorted order's planes) and that many planes hold well
  // under 2^15 particles at the mean density; else 32-bit indices
  const int slow = cfg.dim - 1;
  const double per_plane = (double)c0.n / (double)c0.nc[slow];
  const double reach = 1.5 * (double)(c0.vrad[slow] + 1) * per_plane;
  return (c0.n <= 32768 || reach <= 32767.0) ? 1 : 2;
}

void launch_verlet_lean(const LaunchCtx& L, Buffers b, const int* cellid, const int* start) {
  if (L.dim == 3) {
    if (L.lean == 2) verlet_lean_t<3, true>(L, b, cellid, start);
    else verlet_lean_t<3, false>(L, b, cellid, start);
  } else {
    if (L.lean == 2) verlet_lean_t<2, true>(L, b, cellid, start);
    else verlet_lean_t<2, false>(L, b, cellid, start);
  }
  count_launch(L);
}

void launch_forward_lean(const LaunchCtx& L, Buffers b, float4* R4, const int* cellid,
                         const int* start, unsigned long long* edgecnt, const float* g_arr,
                         bool apply_bc, int phases) {
  if (phases & 1) cudaMemsetAsync(edgecnt, 0, sizeof(unsigned long long), L.stream);
  if (L.dim == 3) {
    if (L.kernel == SPH_KERNEL_QSK)
      forward_lean_k<3, 0>(L, b, R4, cellid, start, edgecnt, g_arr, apply_bc, phases);
    else
      forward_lean_k<3, 1>(L, b, R4, cellid, start, edgecnt, g_arr, apply_bc, phases);
  } else {
    if (L.kernel == SPH_KERNEL_QSK)
      forward_lean_k<2, 0>(L, b, R4, cellid, start, edgecnt, g_arr, apply_bc, phases);
    else
      forward_lean_k<2, 1>(L, b, R4, cellid, start, edgecnt, g_arr, apply_bc, phases);
  }
}

}  // namespace sph
