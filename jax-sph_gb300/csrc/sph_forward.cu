// WCSPH forward pass (jax_sph/solver.py:705-949) as cell-tiled passes over
// particles in cell-sorted order, one thread per receiving particle:
//
//   density pass  walks the 3^d neighbour cells once, keeps exactly the
//                 reference's edges (receiver i, sender j) with
//                 metric(r_j, r_i) < cutoff_sq, records them in a per-step
//                 neighbour list, and computes summation (solver.py:176-178) /
//                 SPH continuity (:24-30) / Riemann continuity (:108-164)
//                 density, EOS (:801-802) and the Shepard wall velocity of
//                 the Riemann wall BC (:547-552); counts edges.
//   wall pass     generalized wall BC of the SPH solver (:431-530) on wall
//                 particles, after every fluid pressure is known.
//   force pass    standard (:221-256) or Riemann (:316-401) acceleration,
//                 transport-velocity acceleration (:199-213), artificial
//                 viscosity (:404-428), g_ext (:936) and, in a step, bc_fn.
//
// The wall and force passes read the neighbour list; a particle with more
// neighbours than the list holds walks the cells again instead. Pair sums are
// accumulated per receiver in registers in a fixed order (deterministic, no
// atomics on physics values). Self pairs contribute exactly zero to every
// gradient sum (dW/dr(0) = 0), so the list omits them.
#include "sph_pairs.cuh"

namespace sph {

namespace {

constexpr int kBlock = 256;
constexpr unsigned kFull = 0xffffffffu;

inline int nblocks(long long n, int b = kBlock) { return (int)((n + b - 1) / b); }

// Per-case edge counter for the NEIGHBOR_LIST_OVERFLOW test: one reduction
// and one atomic per case present in the warp (cases are contiguous, so
// usually one).
__device__ __forceinline__ void count_edges(int ci, int cnt, bool valid,
                                            unsigned long long* edgecnt, const CaseDev* cases,
                                            unsigned* status) {
  const unsigned mask = __ballot_sync(kFull, valid);
  if (!valid) return;
  const int lane = threadIdx.x & 31;
  unsigned remaining = mask;
  while (remaining) {
    const int leader = __ffs(remaining) - 1;
    const int lci = __shfl_sync(mask, ci, leader);
    const unsigned grp = __ballot_sync(mask, ci == lci);
    const unsigned tot = __reduce_add_sync(mask, ci == lci ? (unsigned)cnt : 0u);
    if (lane == leader) {
      unsigned long long old = atomicAdd(&edgecnt[lci], (unsigned long long)tot);
      if ((long long)(old + tot) > cases[lci].edge_cap)
        atomicOr(status, SPH_NEIGHBOR_LIST_OVERFLOW);
    }
    remaining &= ~grp;
  }
}

// ------------------------------------------------------------------ Verlet lists
// Candidate senders of every receiver at the current binning: the particles
// within the Verlet radius (shifted squared distance < v_r2; in a case
// without the fast test, the reference's own edges), self excluded, staged in
// shared memory and written out k-major (coalesced). SORT keeps them in
// ascending original index (insertion while walking), so that every pair sum
// built on them runs in an order that depends neither on the binning nor on
// when it was rebuilt; otherwise they stay in walk (cell) order.
template <int DIM, bool SORT>
__global__ void __launch_bounds__(128)
k_verlet(long long N, Buffers b, const CaseDev* cases, const int* cellid, const int* start,
         int* vl, int* vcnt, int kv) {
  // staging: senders [kv][blockDim] (SORT: and their keys [kv][blockDim])
  extern __shared__ int s_v[];
  const int tid = threadIdx.x, bs = blockDim.x;
  int* js = s_v;
  int* keys = s_v + kv * bs;
  const long long i = blockIdx.x * (long long)bs + tid;
  if (i >= N) return;
  if (tag_of(b.META[i]) == PAD) {  // padding has no candidates
    vcnt[i] = 0;
    return;
  }
  const CaseDev& c = cases[case_of(b.META[i])];
  const float4 ri = b.P4[i];
  int m = 0;
  auto insert = [&](int j) {  // SORT: insertion by original index
    if (m < kv) {
      const int key = b.ORIG[j];
      int p = m;
      while (p > 0 && keys[(p - 1) * bs + tid] > key) {
        keys[p * bs + tid] = keys[(p - 1) * bs + tid];
        js[p * bs + tid] = js[(p - 1) * bs + tid];
        --p;
      }
      keys[p * bs + tid] = key;
      js[p * bs + tid] = j;
    }
    ++m;
  };
  const int cell = cellid[i] - c.cell_off;
  if (c.fast) {
    const float r2 = c.v_r2;
    walk_rows<DIM, true>(c, cell, ri, start, c.vrad, r2, [&](int j0, int j1, float3 s) {
      const float qx = ri.x - s.x, qy = ri.y - s.y, qz = ri.z - s.z;
      if (SORT) {
        for (int j = j0; j < j1; ++j) {
          const float4 rj = __ldg(b.P4 + j);
          const float dx = qx - rj.x, dy = qy - rj.y, dz = (DIM == 3) ? qz - rj.z : 0.f;
          if (j != i && dx * dx + dy * dy + dz * dz < r2) insert(j);
        }
      } else {
        // two gathers per iteration, predicated count, unconditional store
        for (int j = j0; j < j1; j += 2) {
          const bool v1 = j + 1 < j1;
          const float4 ra = __ldg(b.P4 + j);
          const float4 rb = v1 ? __ldg(b.P4 + j + 1) : make_float4(3e30f, 3e30f, 3e30f, 0.f);
          float dx = qx - ra.x, dy = qy - ra.y, dz = (DIM == 3) ? qz - ra.z : 0.f;
          const bool ea = j != i && dx * dx + dy * dy + dz * dz < r2;
          dx = qx - rb.x;
          dy = qy - rb.y;
          dz = (DIM == 3) ? qz - rb.z : 0.f;
          const bool eb = v1 && j + 1 != i && dx * dx + dy * dy + dz * dz < r2;
          js[(m < kv ? m : kv - 1) * bs + tid] = j;
          m += ea;
          js[(m < kv ? m : kv - 1) * bs + tid] = j + 1;
          m += eb;
        }
      }
    });
  } else {
    walk_rows<DIM, false>(c, cell, ri, start, c.vrad, 0.f, [&](int j0, int j1, float3) {
      for (int j = j0; j < j1; ++j) {
        if (j == i || !is_edge<DIM>(ri, __ldg(b.P4 + j), c)) continue;
        if (SORT) {
          insert(j);
        } else {
          if (m < kv) js[m * bs + tid] = j;
          ++m;
        }
      }
    });
  }
  vcnt[i] = m;
  const int e = m < kv ? m : kv;
  for (int k = 0; k < e; ++k) vl[(long long)k * N + i] = js[k * bs + tid];
}

// ------------------------------------------------------------------ density pass
// Two phases per receiver i. (1) Walk the 3^d neighbour cells with the cheap
// membership test and stage the senders in shared memory (k-major, bank
// conflict free); the warp stays converged because the loop body is tiny.
// (2) Loop over the staged senders -- the same count for most lanes -- to
// evaluate the pair physics, copying the list to global memory (coalesced,
// k-major) for the wall and force passes.
//
// MODE 0: summation (fluid receivers), 1: SPH continuity, 2: Riemann
// continuity (fluid receivers), 3: the neighbour list only (delta-SPH
// density evolution follows). `rie_shepard`: wall receivers compute the
// Shepard average of fluid velocities instead (gwbc_fn_riemann_wrapper,
// solver.py:547-552); `sph_gwbc`: the SPH wall BC follows, which ends with
// rho = EOS^-1(p) for every particle (solver.py:516).
template <int DIM, int KER, int MODE, bool KAHAN>
__global__ void __launch_bounds__(kBlock, 4)
k_density(long long N, Buffers b, const CaseDev* cases, const int* cellid, const int* start,
          int mask_self, int rie_shepard, int sph_gwbc, const float* g_arr, float4* R4,
          float4* UT4, NList nl, unsigned long long* edgecnt, unsigned* status) {
  extern __shared__ int s_nbr[];  // [kListSlots][blockDim.x]
  const int tid = threadIdx.x;
  const int bs = blockDim.x;
  long long i = blockIdx.x * (long long)blockDim.x + tid;
  bool valid = i < N;
  int ci = 0, cnt = 0;
  if (valid) {
    const int meta = b.META[i];
    ci = case_of(meta);
    const CaseDev& c = cases[ci];
    const int tag = tag_of(meta);
    const bool fluid = tag == FLUID;
    const float4 ri = b.P4[i];
    // the self pair is always an edge (metric(r, r) = 0 < cutoff^2)
    const bool self_term = !mask_self;
    Acc<KAHAN> s0, sx, sy, sz;
    // the self pair: W(0) in a summation; zero gradient elsewhere; a wall is
    // not a fluid sender of its own Shepard average
    if (MODE == 0 && fluid && self_term) s0.add(kw<KER>(0.f, c));
    // a summation needs only W(|r_ij|): it is accumulated while filtering,
    // in the same order as a second pass would
    const bool sum_here = MODE == 0 && fluid;
    // phase 1: filter the Verlet candidates (ascending original index)
    int m = 0;
    const int kmax = nl.kmax;
    const float lo = c.cut_lo, hi = c.cut_hi;
    const CaseDev* cp = cases + ci;
    const int vc = nl.vcnt[i];
    if (vc <= nl.kv) {
      // two candidates per iteration, software pipelined: the next pair's
      // positions and the pair after's indices are in flight while a pair
      // is tested; predicated count and an unconditional shared-memory store
      const int* vli = nl.vl + i;
      auto cand = [&](int k, int dflt) { return k < vc ? vli[(long long)k * N] : dflt; };
      int ja = cand(0, (int)i), jb = cand(1, ja);
      int jc = cand(2, ja), jd = cand(3, jc);
      float4 ra = __ldg(b.P4 + ja), rb = __ldg(b.P4 + jb);
      // fast cases decide the candidates in the band around the cutoff after
      // the loop (list slots in a mask; slots past 64 re-tested): a receiver
      // has few, but a warp would otherwise run the reference metric in
      // nearly every iteration for some lane
      unsigned long long band = 0;
      for (int k = 0; k < vc; k += 2) {
        const bool v1 = k + 1 < vc;
        const float4 rc = __ldg(b.P4 + jc), rd = __ldg(b.P4 + jd);
        const int je = cand(k + 4, jc), jf = cand(k + 5, je);
        float d2a, d2b;
        bool ea, eb;
        if (c.fast) {
          float3 dr;
          pair_dr<DIM>(ri, ra, c, dr, d2a);
          pair_dr<DIM>(ri, rb, c, dr, d2b);
          ea = d2a < lo;
          eb = v1 && d2b < lo;
          if (!ea && d2a < hi && k < 64) band |= 1ull << k;
          if (v1 && !eb && d2b < hi && k + 1 < 64) band |= 1ull << (k + 1);
        } else {
          ea = edge_mi_d2<DIM>(ri, ra, lo, hi, c, cp, d2a);
          eb = v1 && edge_mi_d2<DIM>(ri, rb, lo, hi, c, cp, d2b);
        }
        if (sum_here) {
          if (ea) s0.add(kw<KER>(d2a > 0.f ? sqrtf(d2a) : 0.f, c));
          if (eb) s0.add(kw<KER>(d2b > 0.f ? sqrtf(d2b) : 0.f, c));
        }
        s_nbr[(m < kmax ? m : kmax - 1) * bs + tid] = ja;
        m += ea;
        s_nbr[(m < kmax ? m : kmax - 1) * bs + tid] = jb;
        m += eb;
        ja = jc;
        jb = jd;
        ra = rc;
        rb = rd;
        jc = je;
        jd = jf;
      }
      // the band's candidates in list order; their edges join the list after
      // the others (W and W' vanish at the cutoff)
      if (c.fast) {
        for (int k = 0; k < vc; ++k) {
          if (k < 64) {
            if (!band) {
              k = 63;  // no more masked slots
              continue;
            }
            k = __ffsll((long long)band) - 1;
            band &= band - 1;
          }
          const int j = vli[(long long)k * N];
          const float4 rj = __ldg(b.P4 + j);
          float3 dr;
          float d2;
          pair_dr<DIM>(ri, rj, c, dr, d2);
          if (k >= 64 && !(!(d2 < lo) && d2 < hi)) continue;
          if (exact_edge<DIM>(ri, rj, cp)) {
            if (sum_here) s0.add(kw<KER>(d2 > 0.f ? sqrtf(d2) : 0.f, c));
            s_nbr[(m < kmax ? m : kmax - 1) * bs + tid] = j;
            ++m;
          }
        }
      }
    } else {
      for_each_edge_slow<DIM>(N, i, ri, c, cp, b.P4, cellid, start, nl,
                              [&](int j, const float4&, const float3&, float d2) {
                                if (sum_here) s0.add(kw<KER>(d2 > 0.f ? sqrtf(d2) : 0.f, c));
                                s_nbr[(m < kmax ? m : kmax - 1) * bs + tid] = j;
                                ++m;
                              });
    }
    cnt = tag == PAD ? 0 : m + (self_term ? 1 : 0);
    nl.cnt[i] = m;

    // phase 2: pair physics over the senders
    const float4 Ui = b.U4[i];
    const float3 ui = f3(Ui);
    const float rho_i = Ui.w;
    const float p_i = b.V4[i].w;
    const bool shepard = rie_shepard && !fluid;
    const bool need_pairs = MODE == 1 || (fluid && MODE == 2) || shepard;
    float3 gi = make_float3(0.f, 0.f, 0.f);
    if (MODE == 2) gi = g_ext<DIM>(c, ri, g_arr, b.ORIG[i]);
    auto pair = [&](int j, const float4& rj, const float3& dr, float d2) {
      const float dist = d2 > 0.f ? sqrtf(d2) : 0.f;
      if (shepard) {
        if (tag_of(b.META[j]) == FLUID) {
          const float w = kw<KER>(dist, c);
          const float4 Uj = b.U4[j];
          s0.add(w);
          sx.add(w * Uj.x);
          sy.add(w * Uj.y);
          sz.add(w * Uj.z);
        }
        return;
      }
      const float4 Uj = b.U4[j];
      const float3 uj = f3(Uj);
      const float inv = 1.0f / (dist + kEps);
      const float gw = kdw<KER>(dist, c);
      if (MODE == 1) {
        const float g = gw * inv;
        const float vj = rj.w / Uj.w;
        s0.add(vj * g * ((ui.x - uj.x) * dr.x + (ui.y - uj.y) * dr.y + (ui.z - uj.z) * dr.z));
        return;
      }
      // MODE 2, fluid receiver (rho_evol_riemann_fn, solver.py:108-164)
      const int tj = tag_of(b.META[j]);
      const float3 e = make_float3(dr.x * inv, dr.y * inv, dr.z * inv);
      const float3 kg = make_float3(gw * e.x, gw * e.y, gw * e.z);
      float uL, uR, pR, rhoR;
      if (is_wall(tj)) {
        const float3 nj = f3(b.NW4[j]);
        uL = -dot3(ui, nj);
        uR = -uL + 2.0f * dot3(uj, nj);
        pR = p_i + rho_i * (-dot3(gi, dr));
        rhoR = eos_rho(pR, c);
      } else {
        uL = -dot3(ui, e);
        uR = -dot3(uj, e);
        pR = b.V4[j].w;
        rhoR = Uj.w;
      }
      const float Uavg = 0.5f * (uL + uR);
      const float rho_avg = 0.5f * (rho_i + rhoR);
      const float Ustar = Uavg + 0.5f * (p_i - pR) / (rho_avg * c.c_ref);
      // v* = U*(-e) + (v_avg - U_avg(-e)),  v_avg = (u_i + u_j)/2
      const float3 vstar = make_float3(-Ustar * e.x + (0.5f * (ui.x + uj.x) + Uavg * e.x),
                                       -Ustar * e.y + (0.5f * (ui.y + uj.y) + Uavg * e.y),
                                       -Ustar * e.z + (0.5f * (ui.z + uj.z) + Uavg * e.z));
      const float3 dv = make_float3(ui.x - vstar.x, ui.y - vstar.y, ui.z - vstar.z);
      s0.add(2.0f * rho_i * rj.w / Uj.w * dot3(dv, kg));
    };
    if (m <= kmax) {
      if (!need_pairs) {
        for (int k = 0; k < m; ++k) nl.nbr[(long long)k * N + i] = s_nbr[k * bs + tid];
      } else {
        int jn = m > 0 ? s_nbr[tid] : 0;
        float4 rn = m > 0 ? __ldg(b.P4 + jn) : ri;
        for (int k = 0; k < m; ++k) {
          const int j = jn;
          const float4 rj = rn;
          if (k + 1 < m) {
            jn = s_nbr[(k + 1) * bs + tid];
            rn = __ldg(b.P4 + jn);
          }
          nl.nbr[(long long)k * N + i] = j;
          float3 dr;
          float d2;
          pair_dr<DIM>(ri, rj, c, dr, d2);
          pair(j, rj, dr, d2);
        }
      }
    } else if (need_pairs) {
      // more senders than list slots: filter the candidates again (the wall
      // and force passes do the same for this receiver)
      for_each_edge_slow<DIM>(N, i, ri, c, cp, b.P4, cellid, start, nl, pair);
    }
    // MODE 3 writes the neighbour list only: the delta-SPH passes compute
    // the density
    if constexpr (MODE != 3) {
      float rho_new = rho_i, drhodt = 0.f;
      if (MODE == 0) {
        // a summation leaves drho/dt as the state had it (solver.py:794-796)
        drhodt = b.A4[i].w;
        if (fluid) rho_new = ri.w * s0.s;
      } else if (MODE == 1) {
        drhodt = rho_i * s0.s;
        rho_new = rho_i + c.dt_rho * drhodt;
      } else {
        if (fluid) drhodt = s0.s;
        rho_new = rho_i + c.dt_rho * drhodt;
      }
      if (UT4) {
        if (shepard) {
          const float den = s0.s + kEps;
          UT4[i] = make_float4(sx.s / den, sy.s / den, sz.s / den, 0.f);
        } else {
          UT4[i] = make_float4(ui.x, ui.y, ui.z, 0.f);
        }
      }
      float p_new = eos_p(rho_new, c);
      if (sph_gwbc && fluid) rho_new = eos_rho(p_new, c);
      R4[i] = make_float4(rho_new, p_new, drhodt, b.ETA[i]);
      if (!isfinite(rho_new) || !isfinite(p_new)) atomicOr(status, SPH_ERR_NONFINITE);
    }
  }
  count_edges(ci, cnt, valid, edgecnt, cases, status);
}

// ------------------------------------------------------------------ wall pass
// gwbc_fn (solver.py:431-530) for wall receivers: Shepard sums over fluid
// senders of u, v, p and rho*dr; writes u, v (U4/V4 xyz) and R4 (rho, p).
// HEAT: also the wall temperature, the Shepard average of the fluid
// temperatures on SOLID_WALL and MOVING_WALL (:518-526; the Riemann solver's
// heat_bc, :556-565, is the same sum: FULL = false runs it alone).
template <int DIM, int KER, bool KAHAN, bool FULL, bool HEAT>
__global__ void __launch_bounds__(kBlock, 4)
k_wall(long long N, Buffers b, const CaseDev* cases, const int* cellid, const int* start,
       int free_slip, const float* g_arr, float4* R4, NList nl) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int meta = b.META[i];
  if (!is_wall(tag_of(meta))) return;
  const CaseDev& c = cases[case_of(meta)];
  const float4 ri = b.P4[i];
  Acc<KAHAN> sw, su[3], sv[3], sp, sr[3], sT;
  for_each_neighbour<DIM>(N, i, ri, c, cases + case_of(meta), b.P4, cellid, start, nl,
                          [&](int j, const float4& rj, const float3& dr, float d2) {
    if (tag_of(b.META[j]) != FLUID) return;
    const float dist = d2 > 0.f ? sqrtf(d2) : 0.f;
    const float w = kw<KER>(dist, c);
    sw.add(w);
    if (HEAT) sT.add(w * b.TH4[j].x);
    if (!FULL) return;
    const float4 Uj = b.U4[j], Vj = b.V4[j], Rj = R4[j];
    su[0].add(w * Uj.x); su[1].add(w * Uj.y); su[2].add(w * Uj.z);
    sv[0].add(w * Vj.x); sv[1].add(w * Vj.y); sv[2].add(w * Vj.z);
    sp.add(w * Rj.y);
    const float rw = Rj.x * w;
    sr[0].add(rw * dr.x); sr[1].add(rw * dr.y); sr[2].add(rw * dr.z);
  });
  const float den = sw.s + kEps;
  if (HEAT && tag_of(meta) != DIRICHLET_WALL) b.TH4[i].x = sT.s / den;
  if (!FULL) return;
  float3 uw = make_float3(su[0].s / den, su[1].s / den, su[2].s / den);
  float3 vw = make_float3(sv[0].s / den, sv[1].s / den, sv[2].s / den);
  if (free_slip) {
    const float4 nw = b.NW4[i];
    const float3 n = make_float3(-nw.x, -nw.y, -nw.z);
    const float pu = dot3(uw, n), pv = dot3(vw, n);
    uw = make_float3(n.x * pu, n.y * pu, n.z * pu);
    vw = make_float3(n.x * pv, n.y * pv, n.z * pv);
  }
  const float4 Ui = b.U4[i], Vi = b.V4[i];
  b.U4[i] = make_float4(2.f * Ui.x - uw.x, 2.f * Ui.y - uw.y, 2.f * Ui.z - uw.z, Ui.w);
  b.V4[i] = make_float4(2.f * Vi.x - vw.x, 2.f * Vi.y - vw.y, 2.f * Vi.z - vw.z, Vi.w);
  const float3 gi = g_ext<DIM>(c, ri, g_arr, b.ORIG[i]);
  const float pw = (sp.s + (gi.x * sr[0].s + gi.y * sr[1].s + gi.z * sr[2].s)) / den;
  const float4 Ri = R4[i];
  R4[i] = make_float4(eos_rho(pw, c), pw, Ri.z, Ri.w);
}

// ------------------------------------------------------------------ heat pass
// Heat conduction (solver.py:832-850): the temperature first takes the rate
// it came with, T' = T + dt dT/dt (walls after the wall temperature BC),
// then the new rate (temperature_derivative_wrapper, :591-610)
//   dT/dt_i = sum_j 4 m_j kappa_ij (T'_i - T'_j) F_ij / (Cp_i rho_i rho_j),
//   kappa_ij = kappa_i kappa_j / (kappa_i + kappa_j),
//   F_ij = r_ij . grad W_ij / (d^2 + eps),
// on the densities after the density passes and the wall BC. Writes
// (T', dT/dt) to TO; the state takes them when it folds the forward result.
template <int DIM, int KER, bool KAHAN>
__global__ void __launch_bounds__(kBlock)
k_heat(long long N, Buffers b, const CaseDev* cases, const int* cellid, const int* start,
       const float4* R4, NList nl) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int ci = case_of(b.META[i]);
  const CaseDev& c = cases[ci];
  const float4 ri = b.P4[i];
  const float4 ti = b.TH4[i];
  const float Ti = ti.x + c.dt_rho * ti.y;
  const float rho_i = R4[i].x;
  Acc<KAHAN> s;
  for_each_neighbour<DIM>(N, i, ri, c, cases + ci, b.P4, cellid, start, nl,
                          [&](int j, const float4& rj, const float3& dr, float d2) {
    const float dist = d2 > 0.f ? sqrtf(d2) : 0.f;
    const float4 tj = b.TH4[j];
    const float Tj = tj.x + c.dt_rho * tj.y;
    const float g = kdw<KER>(dist, c) / (dist + kEps);
    const float F = g * (dr.x * dr.x + dr.y * dr.y + dr.z * dr.z) / (dist * dist + kEps);
    const float keff = ti.z * tj.z / (ti.z + tj.z);
    s.add(4.0f * rj.w * keff * (Ti - Tj) * F / (ti.w * rho_i * R4[j].x));
  });
  b.TO[i] = make_float2(Ti, s.s);
}

// ------------------------------------------------------------------ force pass
// SOLVER 0: standard SPH with transport-velocity stress; 1: Riemann SPH;
// 2: delta-SPH (standard plus the diffusive term).
// The per-pair quotients use the fast division intrinsic (at most 2 ulp, for
// denominators far inside its range): the correctly rounded division is a
// multi-instruction sequence that cost a quarter of this pass, and the
// float32 tolerances against the float64 oracle hold either way.
template <int DIM, int KER, int SOLVER, bool KAHAN>
__global__ void __launch_bounds__(kBlock, 3)
k_force(long long N, Buffers b, const CaseDev* cases, const int* cellid, const int* start,
        int bc_trick, int free_slip, const float* g_arr, const float4* R4, const float4* UT4,
        NList nl, bool apply_bc, unsigned* status) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int meta = b.META[i];
  const CaseDev& c = cases[case_of(meta)];
  const int tag = tag_of(meta);
  const bool fluid_i = tag == FLUID;
  const float4 ri = b.P4[i];
  const float m_i = ri.w;
  const float3 ui = f3(b.U4[i]);
  const float3 vi = f3(b.V4[i]);
  const float4 Ri = R4[i];
  const float rho_i = Ri.x, p_i = Ri.y, eta_i = Ri.w;
  const float Vi = m_i / rho_i;
  const float Vi2 = Vi * Vi;
  const float inv_mi = 1.0f / m_i;
  // A_i r = rho_i u_i ((v_i - u_i) . r)  (tvf_stress_fn, solver.py:216-218)
  const float3 Ai = make_float3(rho_i * ui.x, rho_i * ui.y, rho_i * ui.z);
  const float3 wi = make_float3(vi.x - ui.x, vi.y - ui.y, vi.z - ui.z);
  const float3 gi = g_ext<DIM>(c, ri, g_arr, b.ORIG[i]);
  const bool av = c.av_alpha != 0.0f;
  const float mask_i = (SOLVER == 1 && bc_trick && free_slip) ? (fluid_i ? 1.f : 0.f) : 1.f;
  Acc<KAHAN> ax, ay, az, tx, ty, tz;
  auto pair = [&](int j, const float4& rj, const float4& Uj4, const float4& Vj4,
                  const float4& Rj, const float3& dr, float d2) {
    const float dist = d2 > 0.f ? sqrtf(d2) : 0.f;
    const float gw = kdw<KER>(dist, c);
    const float inv_d = __fdividef(1.0f, dist + kEps);
    const float rho_j = Rj.x, p_j = Rj.y, eta_j = Rj.w, m_j = rj.w;
    const float Vj = __fdividef(m_j, rho_j);
    const float cc = (Vi2 + Vj * Vj) * inv_mi * gw * inv_d;
    const float3 uj = f3(Uj4);
    const float eta_ij = __fdividef(2.f * eta_i * eta_j, eta_i + eta_j + kEps);
    int tj = FLUID;
    if (SOLVER != 0 || av) tj = tag_of(b.META[j]);
    float3 a;
    if (SOLVER != 1) {
      const float3 vj = f3(Vj4);
      const float p_ij = __fdividef(rho_j * p_i + rho_i * p_j, rho_i + rho_j);
      const float ki = dot3(wi, dr);
      const float kj = dot3(make_float3(vj.x - uj.x, vj.y - uj.y, vj.z - uj.z), dr);
      const float3 Ar = make_float3(0.5f * (Ai.x * ki + rho_j * uj.x * kj),
                                    0.5f * (Ai.y * ki + rho_j * uj.y * kj),
                                    0.5f * (Ai.z * ki + rho_j * uj.z * kj));
      a = make_float3(cc * (-p_ij * dr.x + Ar.x + eta_ij * (ui.x - uj.x)),
                      cc * (-p_ij * dr.y + Ar.y + eta_ij * (ui.y - uj.y)),
                      cc * (-p_ij * dr.z + Ar.z + eta_ij * (ui.z - uj.z)));
      if (SOLVER == 2 && tj == FLUID) {
        // delta-SPH diffusion (solver.py:293-309): V_j pi_ij W'(d) e_ij
        // alpha h c_ref rho_ref / rho_i, pi_ij = (u_j - u_i).(-r_ij) / (d + eps)^2
        const float pi_ij = ((uj.x - ui.x) * -dr.x + (uj.y - ui.y) * -dr.y +
                             (uj.z - ui.z) * -dr.z) * inv_d * inv_d;
        const float k = Vj * pi_ij * gw * inv_d * __fdividef(c.delta_coef, rho_i);
        a.x += k * dr.x;
        a.y += k * dr.y;
        a.z += k * dr.z;
      }
    } else {
      const float3 e = make_float3(dr.x * inv_d, dr.y * inv_d, dr.z * inv_d);
      const float3 kg = make_float3(gw * e.x, gw * e.y, gw * e.z);
      const bool wj = is_wall(tj);
      float uL, uR, pR, rhoR;
      float3 ud = uj;
      if (wj) {
        const float3 nj = f3(b.NW4[j]);
        uL = -dot3(ui, nj);
        uR = -uL + 2.f * dot3(uj, nj);
        pR = p_i + rho_i * (-dot3(gi, dr));
        rhoR = eos_rho(pR, c);
        const float4 ut = UT4[j];
        ud = make_float3(2.f * uj.x - ut.x, 2.f * uj.y - ut.y, 2.f * uj.z - ut.z);
      } else {
        uL = -dot3(ui, e);
        uR = -dot3(uj, e);
        pR = p_j;
        rhoR = rho_j;
      }
      const float P_avg = 0.5f * (p_i + pR);
      const float rho_avg = 0.5f * (rho_i + rhoR);
      float beta;
      if (c.eta_limiter == -1.0f) {
        beta = c.c_ref;
      } else {
        beta = fminf(c.eta_limiter * fmaxf(uL - uR, 0.f), c.c_ref);
      }
      const float Pstar = P_avg + 0.5f * rho_avg * (uL - uR) * beta;
      const float rr = rho_i * rho_j;
      const float k9 = -2.f * m_j * __fdividef(Pstar, rr);
      const float k6 = 2.f * m_j * __fdividef(eta_ij, rr) * inv_d * gw * mask_i;
      a = make_float3(k9 * kg.x + k6 * (ui.x - ud.x), k9 * kg.y + k6 * (ui.y - ud.y),
                      k9 * kg.z + k6 * (ui.z - ud.z));
    }
    if (av && fluid_i && tj == FLUID) {
      const float rho_ab = 0.5f * (rho_i + rho_j);
      const float num = m_j * c.av_alpha * c.av_hab * c.av_cab *
                        ((ui.x - uj.x) * dr.x + (ui.y - uj.y) * dr.y + (ui.z - uj.z) * dr.z);
      const float k = num * gw * inv_d / (rho_ab * (dist * dist + c.av_eps));
      a.x += k * dr.x;
      a.y += k * dr.y;
      a.z += k * dr.z;
    }
    ax.add(a.x);
    ay.add(a.y);
    az.add(a.z);
    // acceleration_tvf_fn: c * p_bg_i * r_ij
    const float ct = cc * c.p_bg_tvf;
    tx.add(ct * dr.x);
    ty.add(ct * dr.y);
    tz.add(ct * dr.z);
  };
  const int m = nl.cnt[i];
  if (m <= nl.kmax) {
    // the next sender's four records are loaded while the current pair is
    // evaluated, and its index one step earlier still
    const int* nbi = nl.nbr + i;
    int j = m > 0 ? nbi[0] : (int)i;
    int jn = m > 1 ? nbi[N] : j;
    float4 rj = __ldg(b.P4 + j), uj = __ldg(b.U4 + j), vj = __ldg(b.V4 + j), Rj = __ldg(R4 + j);
    for (int k = 0; k < m; ++k) {
      const int jc = j;
      const float4 rc = rj, uc = uj, vc = vj, Rc = Rj;
      j = jn;
      if (k + 2 < m) jn = nbi[(long long)(k + 2) * N];
      if (k + 1 < m) {
        rj = __ldg(b.P4 + j);
        uj = __ldg(b.U4 + j);
        vj = __ldg(b.V4 + j);
        Rj = __ldg(R4 + j);
      }
      float3 dr;
      float d2;
      pair_dr<DIM>(ri, rc, c, dr, d2);
      pair(jc, rc, uc, vc, Rc, dr, d2);
    }
  } else {
    for_each_edge_slow<DIM>(N, i, ri, c, cases + case_of(meta), b.P4, cellid, start, nl,
                            [&](int j, const float4& rj, const float3& dr, float d2) {
                              pair(j, rj, b.U4[j], b.V4[j], R4[j], dr, d2);
                            });
  }
  float3 dudt = make_float3(ax.s + gi.x, ay.s + gi.y, az.s + gi.z);
  float3 dvdt = make_float3(tx.s, ty.s, tz.s);
  if (DIM == 2) {
    dudt.z = 0.f;
    dvdt.z = 0.f;
  }
  if (apply_bc) {
    dudt = bc_acc(dudt, tag, c);
    dvdt = bc_acc(dvdt, tag, c);
  }
  if (!isfinite(dudt.x) || !isfinite(dudt.y) || !isfinite(dudt.z)) atomicOr(status, SPH_ERR_NONFINITE);
  b.A4[i] = make_float4(dudt.x, dudt.y, dudt.z, Ri.z);
  b.A2[i] = make_float4(dvdt.x, dvdt.y, dvdt.z, 0.f);
}

template <int DIM, int KER, bool KAHAN>
void forward_t(const LaunchCtx& L, Buffers b, float4* R4, float4* UT4, const int* cellid,
               const int* start, unsigned long long* edgecnt, const float* g_arr, bool apply_bc,
               bool has_walls, int phases) {
  const int bt = L.block > 0 ? L.block : kBlock;
  const int g = nblocks(L.N, bt);
  const size_t smem = sizeof(int) * kListSlots * bt;
  cudaStream_t st = L.stream;
  const bool rie = L.solver == SPH_SOLVER_RIE;
  const int rie_shepard = rie && L.bc_trick && !L.free_slip;
  const int sph_gwbc = !rie && L.bc_trick;
  float4* ut = rie ? UT4 : nullptr;
  NList nl{L.nbr, L.nbr_cnt, L.kmax, L.vl, L.vcnt, L.kv, L.rref};
  // with renormalisation the evolved density goes to R4e first; the wall
  // BC's rho = EOS^-1(p) then follows the renormalisation
  if (phases & 1) {
    const bool renorm = L.rho_evol && L.rho_renorm;
    float4* Rd = renorm ? L.R4e : R4;
    const int gw_d = renorm ? 0 : sph_gwbc;
  #define SPH_DENSITY(MODE)                                                                 \
    k_density<DIM, KER, MODE, KAHAN><<<g, bt, smem, st>>>(L.N, b, L.cases, cellid, start,  \
                                                           L.mask_self, rie_shepard,        \
                                                           gw_d, g_arr, Rd, ut, nl,         \
                                                           edgecnt, L.status)
    if (!L.rho_evol)
      SPH_DENSITY(0);
    else if (rie)
      SPH_DENSITY(2);
    else if (L.solver == SPH_SOLVER_DELTA)
      SPH_DENSITY(3);
    else
      SPH_DENSITY(1);
  #undef SPH_DENSITY
    count_launch(L);
    if (L.rho_evol && L.solver == SPH_SOLVER_DELTA)
      launch_delta_density(L, b, Rd, cellid, start, gw_d);
    if (renorm) launch_renorm(L, b, Rd, R4, cellid, start, sph_gwbc);
    mark(L, 2);
    if (sph_gwbc && has_walls) {
      if (L.heat)
        k_wall<DIM, KER, KAHAN, true, true><<<g, bt, 0, st>>>(L.N, b, L.cases, cellid, start,
                                                              L.free_slip, g_arr, R4, nl);
      else
        k_wall<DIM, KER, KAHAN, true, false><<<g, bt, 0, st>>>(L.N, b, L.cases, cellid, start,
                                                               L.free_slip, g_arr, R4, nl);
      count_launch(L);
    } else if (L.heat && rie && L.bc_trick && has_walls) {
      k_wall<DIM, KER, KAHAN, false, true><<<g, bt, 0, st>>>(L.N, b, L.cases, cellid, start,
                                                             L.free_slip, g_arr, R4, nl);
      count_launch(L);
    }
    if (L.heat) {
      k_heat<DIM, KER, KAHAN><<<g, bt, 0, st>>>(L.N, b, L.cases, cellid, start, R4, nl);
      count_launch(L);
    }
    mark(L, 3);
  }
  if (!(phases & 2)) return;
  if (rie)
    k_force<DIM, KER, 1, KAHAN><<<g, bt, 0, st>>>(L.N, b, L.cases, cellid, start,
                                                        L.bc_trick, L.free_slip, g_arr, R4, UT4,
                                                        nl, apply_bc, L.status);
  else if (L.solver == SPH_SOLVER_DELTA)
    k_force<DIM, KER, 2, KAHAN><<<g, bt, 0, st>>>(L.N, b, L.cases, cellid, start,
                                                        L.bc_trick, L.free_slip, g_arr, R4,
                                                        nullptr, nl, apply_bc, L.status);
  else
    k_force<DIM, KER, 0, KAHAN><<<g, bt, 0, st>>>(L.N, b, L.cases, cellid, start,
                                                        L.bc_trick, L.free_slip, g_arr, R4,
                                                        nullptr, nl, apply_bc, L.status);
  count_launch(L);
  mark(L, 4);
}

template <int DIM, int KER>
void forward_k(const LaunchCtx& L, Buffers b, float4* R4, float4* UT4, const int* cellid,
               const int* start, unsigned long long* edgecnt, const float* g_arr, bool apply_bc,
               bool has_walls, int phases) {
  if (L.kahan)
    forward_t<DIM, KER, true>(L, b, R4, UT4, cellid, start, edgecnt, g_arr, apply_bc, has_walls,
                              phases);
  else
    forward_t<DIM, KER, false>(L, b, R4, UT4, cellid, start, edgecnt, g_arr, apply_bc, has_walls,
                               phases);
}

}  // namespace

cudaError_t prepare_kernels(int /*kv*/) {
  // the attribute belongs to the kernel, not to a handle: allow the largest
  // staging any handle uses (kv * verlet_block(kv) <= 96 * 128 for every kv)
  const int most = 96 * 128 * (int)sizeof(int);
  cudaError_t e = cudaFuncSetAttribute(k_verlet<3, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * most);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_verlet<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             2 * most);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_verlet<3, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             most);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_verlet<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             most);
  return e;
}

void launch_verlet(const LaunchCtx& L, Buffers b, const int* cellid, const int* start) {
  if (L.lean) {
    launch_verlet_lean(L, b, cellid, start);
    return;
  }
  const int bt = verlet_block(L.kv);
  const int g = nblocks(L.N, bt);
  const size_t smem = (L.canonical ? 2 : 1) * sizeof(int) * L.kv * bt;
  if (L.canonical) {
    if (L.dim == 3)
      k_verlet<3, true><<<g, bt, smem, L.stream>>>(L.N, b, L.cases, cellid, start, L.vl, L.vcnt,
                                                   L.kv);
    else
      k_verlet<2, true><<<g, bt, smem, L.stream>>>(L.N, b, L.cases, cellid, start, L.vl, L.vcnt,
                                                   L.kv);
  } else {
    if (L.dim == 3)
      k_verlet<3, false><<<g, bt, smem, L.stream>>>(L.N, b, L.cases, cellid, start, L.vl, L.vcnt,
                                                    L.kv);
    else
      k_verlet<2, false><<<g, bt, smem, L.stream>>>(L.N, b, L.cases, cellid, start, L.vl, L.vcnt,
                                                    L.kv);
  }
  count_launch(L);
}

void launch_forward(const LaunchCtx& L, Buffers b, const float4* /*R4*/, float4* R4w, float4* UT4,
                    const int* cellid, const int* start, unsigned long long* edgecnt,
                    const float* g_arr, bool apply_bc, bool has_walls, int phases) {
  if (L.lean) {
    launch_forward_lean(L, b, R4w, cellid, start, edgecnt, g_arr, apply_bc, phases);
    return;
  }
  if (phases & 1)
    cudaMemsetAsync(edgecnt, 0, sizeof(unsigned long long) * L.n_cases, L.stream);
  if (L.dim == 3) {
    if (L.kernel == SPH_KERNEL_QSK)
      forward_k<3, 0>(L, b, R4w, UT4, cellid, start, edgecnt, g_arr, apply_bc, has_walls, phases);
    else
      forward_k<3, 1>(L, b, R4w, UT4, cellid, start, edgecnt, g_arr, apply_bc, has_walls, phases);
  } else {
    if (L.kernel == SPH_KERNEL_QSK)
      forward_k<2, 0>(L, b, R4w, UT4, cellid, start, edgecnt, g_arr, apply_bc, has_walls, phases);
    else
      forward_k<2, 1>(L, b, R4w, UT4, cellid, start, edgecnt, g_arr, apply_bc, has_walls, phases);
  }
}

}  // namespace sph
