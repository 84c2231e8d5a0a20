// Neighbour iteration shared by the forward passes: the per-step neighbour
// list written by the density pass, and the Verlet candidates (or a cell walk)
// for a receiver with more neighbours than that list holds.
#pragma once
#include "sph_internal.cuh"

namespace sph {

__device__ __forceinline__ float3 f3(const float4& a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float dot3(const float3& a, const float3& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}

struct NList {
  int* nbr;   // [kmax][N] sender indices (k-major)
  int* cnt;   // [N] neighbours without self (may exceed kmax)
  int kmax;
  const int* vl;   // [kv][N] Verlet candidates, ascending original index
  const int* vcnt; // [N] candidates (may exceed kv)
  int kv;
  const float4* rref;  // positions at the last rebuild
};

// Visit the senders j of receiver i (self excluded) that are edges at the
// current positions, from its Verlet candidates (ascending original index),
// or -- a receiver with more candidates than the list holds -- by walking the
// cells of the last binning around its position at that binning: every
// sender now within the cutoff was within the Verlet radius of it then.
template <int DIM, typename F>
__device__ __forceinline__ void for_each_edge_slow(long long N, long long i, const float4& ri,
                                                   const CaseDev& c, const CaseDev* cp,
                                                   const float4* __restrict__ P4,
                                                   const int* cellid, const int* start,
                                                   const NList& L, F&& f) {
  const float lo = c.cut_lo, hi = c.cut_hi;
  auto test = [&](int j) {
    const float4 rj = __ldg(P4 + j);
    if (edge_mi<DIM>(ri, rj, lo, hi, c, cp)) {
      float3 dr;
      float d2;
      pair_dr<DIM>(ri, rj, c, dr, d2);
      f(j, rj, dr, d2);
    }
  };
  const int vc = L.vcnt[i];
  if (vc <= L.kv) {
    for (int k = 0; k < vc; ++k) test(L.vl[(long long)k * N + i]);
    return;
  }
  const float4 r0 = L.rref[i];
  auto visit = [&](int j0, int j1, float3) {
    for (int j = j0; j < j1; ++j)
      if (j != i) test(j);
  };
  if (c.fast)
    walk_rows<DIM, true>(c, cellid[i] - c.cell_off, r0, start, c.vrad, c.v_r2, visit);
  else
    walk_rows<DIM, false>(c, cellid[i] - c.cell_off, r0, start, c.vrad, 0.f, visit);
}

// Visit the senders j of receiver i (self excluded): from the step's
// neighbour list, or the slow way when it overflowed for i.
template <int DIM, typename F>
__device__ __forceinline__ void for_each_neighbour(long long N, long long i, const float4& ri,
                                                   const CaseDev& c, const CaseDev* cp,
                                                   const float4* __restrict__ P4,
                                                   const int* cellid, const int* start,
                                                   const NList& L, F&& f) {
  const int m = L.cnt[i];
  if (m <= L.kmax) {
    // software pipelined: the next sender's index and position are loaded
    // while the current pair is evaluated
    int jn = m > 0 ? L.nbr[i] : 0;
    float4 rn = m > 0 ? __ldg(P4 + jn) : ri;
    for (int k = 0; k < m; ++k) {
      const int j = jn;
      const float4 rj = rn;
      if (k + 1 < m) {
        jn = L.nbr[(long long)(k + 1) * N + i];
        rn = __ldg(P4 + jn);
      }
      float3 dr;
      float d2;
      pair_dr<DIM>(ri, rj, c, dr, d2);
      f(j, rj, dr, d2);
    }
    return;
  }
  for_each_edge_slow<DIM>(N, i, ri, c, cp, P4, cellid, start, L, f);
}

}  // namespace sph
