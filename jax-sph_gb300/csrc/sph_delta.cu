// Density passes that need more than one sweep over the neighbours:
//
//   delta-SPH density evolution (rho_evol_fn_delta, jax_sph/solver.py:33-105):
//     L pass     M_i = sum_j (-r_ij) (x) grad W_ij V_j, L_i = M_i^-1, and the
//                continuity sum sum_j (u_i - u_j).grad W_ij V_j;
//     grad pass  G_i = L_i sum_j (rho_j - rho_i) grad W_ij V_j and
//                H_i = V_i sum_j (rho_i - rho_j) L_j grad W_ij;
//     rho pass   psi_ij = 2 (rho_j - rho_i)(-r_ij)/(d + eps)^2 - G_i - H_j,
//                drho/dt = rho_i cont_i + c_ref delta h sum_j psi_ij.grad W_ij V_j
//                (fluid senders), rho += dt drho/dt.
//   The reference inverts a second matrix per particle, the sum of
//   r_ij (x) grad W_ij V_i over the edges it sends (L_matj). With r_ji = -r_ij
//   and the same neighbour set that sum is -M_j, so H uses -L_j; the two sets
//   can differ only by pairs at the cutoff distance, where grad W vanishes.
//
//   density renormalisation (rho_renorm_fn, solver.py:167-173):
//     rho_i = sum_j m_j W_ij / min(sum_j (m_j / rho_j) W_ij, 1), self pair
//     included, on the evolved densities.
//
// Every pass is one thread per receiving particle over the step's neighbour
// list (cell-sorted order), sums in registers in list order.
#include "sph_pairs.cuh"

namespace sph {

namespace {

constexpr int kBlock = 256;

inline int nblocks(long long n, int b = kBlock) { return (int)((n + b - 1) / b); }

__device__ __forceinline__ float comp(const float3& v, int a) {
  return a == 0 ? v.x : (a == 1 ? v.y : v.z);
}
__device__ __forceinline__ float comp(const float4& v, int a) {
  return a == 0 ? v.x : (a == 1 ? v.y : v.z);
}

// Scratch planes of N float4 each: 0..2 rows of L, 3 (G, continuity sum), 4 H.
__device__ __forceinline__ float4* plane(float4* D, long long N, int k) { return D + k * N; }

template <int DIM, int KER, bool KAHAN>
__global__ void __launch_bounds__(kBlock)
k_delta_L(long long N, Buffers b, const CaseDev* cases, const int* cellid, const int* start,
          NList nl, float4* D) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int ci = case_of(b.META[i]);
  const CaseDev& c = cases[ci];
  const float4 ri = b.P4[i];
  const float4 Ui = b.U4[i];
  Acc<KAHAN> m[DIM][DIM], cont;
  for_each_neighbour<DIM>(N, i, ri, c, cases + ci, b.P4, cellid, start, nl,
                          [&](int j, const float4& rj, const float3& dr, float d2) {
    const float dist = d2 > 0.f ? sqrtf(d2) : 0.f;
    const float g = kdw<KER>(dist, c) / (dist + kEps);
    const float4 Uj = b.U4[j];
    const float vj = rj.w / Uj.w;
    const float3 kg = make_float3(g * dr.x, g * dr.y, g * dr.z);
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
      for (int e = 0; e < DIM; ++e) m[a][e].add(-comp(dr, a) * (comp(kg, e) * vj));
    cont.add(((Ui.x - Uj.x) * kg.x + (Ui.y - Uj.y) * kg.y + (Ui.z - Uj.z) * kg.z) * vj);
  });
  float4 row[3] = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f),
                   make_float4(0.f, 0.f, 0.f, 0.f)};
  if constexpr (DIM == 2) {
    const float a = m[0][0].s, bb = m[0][1].s, cc = m[1][0].s, d = m[1][1].s;
    const float det = a * d - bb * cc;
    row[0] = make_float4(d / det, -bb / det, 0.f, 0.f);
    row[1] = make_float4(-cc / det, a / det, 0.f, 0.f);
  } else {
    // adjugate over the determinant
    const float m00 = m[0][0].s, m01 = m[0][1].s, m02 = m[0][2].s;
    const float m10 = m[1][0].s, m11 = m[1][1].s, m12 = m[1][2].s;
    const float m20 = m[2][0].s, m21 = m[2][1].s, m22 = m[2][2].s;
    const float c00 = m11 * m22 - m12 * m21, c01 = m12 * m20 - m10 * m22,
                c02 = m10 * m21 - m11 * m20;
    const float det = m00 * c00 + m01 * c01 + m02 * c02;
    row[0] = make_float4(c00 / det, (m02 * m21 - m01 * m22) / det,
                         (m01 * m12 - m02 * m11) / det, 0.f);
    row[1] = make_float4(c01 / det, (m00 * m22 - m02 * m20) / det,
                         (m02 * m10 - m00 * m12) / det, 0.f);
    row[2] = make_float4(c02 / det, (m01 * m20 - m00 * m21) / det,
                         (m00 * m11 - m01 * m10) / det, 0.f);
  }
#pragma unroll
  for (int a = 0; a < DIM; ++a) plane(D, N, a)[i] = row[a];
  plane(D, N, 3)[i] = make_float4(0.f, 0.f, 0.f, cont.s);
}

template <int DIM, int KER, bool KAHAN>
__global__ void __launch_bounds__(kBlock)
k_delta_grad(long long N, Buffers b, const CaseDev* cases, const int* cellid, const int* start,
             NList nl, float4* D) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int ci = case_of(b.META[i]);
  const CaseDev& c = cases[ci];
  const float4 ri = b.P4[i];
  const float rho_i = b.U4[i].w;
  Acc<KAHAN> s[DIM], h[DIM];
  for_each_neighbour<DIM>(N, i, ri, c, cases + ci, b.P4, cellid, start, nl,
                          [&](int j, const float4& rj, const float3& dr, float d2) {
    const float dist = d2 > 0.f ? sqrtf(d2) : 0.f;
    const float g = kdw<KER>(dist, c) / (dist + kEps);
    const float rho_j = b.U4[j].w;
    const float vj = rj.w / rho_j;
    const float3 kg = make_float3(g * dr.x, g * dr.y, g * dr.z);
    const float wi = (rho_j - rho_i) * vj;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      const float4 L = plane(D, N, a)[j];
      const float lk = L.x * kg.x + L.y * kg.y + L.z * kg.z;
      s[a].add(wi * comp(kg, a));
      h[a].add((rho_i - rho_j) * lk);
    }
  });
  float sv[3] = {0.f, 0.f, 0.f}, g[3] = {0.f, 0.f, 0.f}, hv[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int a = 0; a < DIM; ++a) sv[a] = s[a].s;
  const float vi = ri.w / rho_i;
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    const float4 L = plane(D, N, a)[i];
    g[a] = L.x * sv[0] + L.y * sv[1] + L.z * sv[2];
    hv[a] = vi * h[a].s;
  }
  const float cont = plane(D, N, 3)[i].w;
  plane(D, N, 3)[i] = make_float4(g[0], g[1], g[2], cont);
  plane(D, N, 4)[i] = make_float4(hv[0], hv[1], hv[2], 0.f);
}

template <int DIM, int KER, bool KAHAN>
__global__ void __launch_bounds__(kBlock)
k_delta_rho(long long N, Buffers b, const CaseDev* cases, const int* cellid, const int* start,
            NList nl, const float4* D, int sph_gwbc, float4* Rout, unsigned* status) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int meta = b.META[i];
  const int ci = case_of(meta);
  const CaseDev& c = cases[ci];
  const float4 ri = b.P4[i];
  const float rho_i = b.U4[i].w;
  const float4 Gi = D[3 * N + i];
  Acc<KAHAN> diff;
  for_each_neighbour<DIM>(N, i, ri, c, cases + ci, b.P4, cellid, start, nl,
                          [&](int j, const float4& rj, const float3& dr, float d2) {
    if (tag_of(b.META[j]) != FLUID) return;
    const float dist = d2 > 0.f ? sqrtf(d2) : 0.f;
    const float inv = 1.0f / (dist + kEps);
    const float g = kdw<KER>(dist, c) * inv;
    const float rho_j = b.U4[j].w;
    const float vj = rj.w / rho_j;
    const float4 Hj = D[4 * N + j];
    const float t = 2.0f * (rho_j - rho_i) * inv * inv;
    // psi_ij . grad W_ij with psi = t (-r_ij) - G_i - H_j and grad W = g r_ij
    const float px = -t * dr.x - Gi.x - Hj.x, py = -t * dr.y - Gi.y - Hj.y,
                pz = -t * dr.z - Gi.z - Hj.z;
    diff.add((px * (g * dr.x) + py * (g * dr.y) + pz * (g * dr.z)) * vj);
  });
  const float drhodt = rho_i * Gi.w + c.delta_rho_coef * diff.s;
  float rho_new = rho_i + c.dt_rho * drhodt;
  const float p_new = eos_p(rho_new, c);
  if (sph_gwbc && tag_of(meta) == FLUID) rho_new = eos_rho(p_new, c);
  Rout[i] = make_float4(rho_new, p_new, drhodt, b.ETA[i]);
  if (!isfinite(rho_new) || !isfinite(p_new)) atomicOr(status, SPH_ERR_NONFINITE);
}

template <int DIM, int KER, bool KAHAN>
__global__ void __launch_bounds__(kBlock)
k_renorm(long long N, Buffers b, const CaseDev* cases, const int* cellid, const int* start,
         NList nl, const float4* Rin, int mask_self, int sph_gwbc, float4* Rout,
         unsigned* status) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int meta = b.META[i];
  const int ci = case_of(meta);
  const CaseDev& c = cases[ci];
  const float4 ri = b.P4[i];
  const float4 Ri = Rin[i];
  Acc<KAHAN> num, den;
  if (!mask_self) {
    const float w0 = kw<KER>(0.f, c);
    num.add(ri.w * w0);
    den.add(ri.w / Ri.x * w0);
  }
  for_each_neighbour<DIM>(N, i, ri, c, cases + ci, b.P4, cellid, start, nl,
                          [&](int j, const float4& rj, const float3&, float d2) {
    const float w = kw<KER>(d2 > 0.f ? sqrtf(d2) : 0.f, c);
    num.add(rj.w * w);
    den.add(rj.w / Rin[j].x * w);
  });
  float rho = num.s / (den.s > 1.0f ? 1.0f : den.s);
  const float p = eos_p(rho, c);
  if (sph_gwbc && tag_of(meta) == FLUID) rho = eos_rho(p, c);
  Rout[i] = make_float4(rho, p, Ri.z, Ri.w);
  if (!isfinite(rho) || !isfinite(p)) atomicOr(status, SPH_ERR_NONFINITE);
}

template <int DIM, int KER, bool KAHAN>
void delta_t(const LaunchCtx& L, Buffers b, float4* Rout, const int* cellid, const int* start,
             int sph_gwbc) {
  const int bt = kBlock;
  const int g = nblocks(L.N, bt);
  NList nl{L.nbr, L.nbr_cnt, L.kmax, L.vl, L.vcnt, L.kv, L.rref};
  k_delta_L<DIM, KER, KAHAN><<<g, bt, 0, L.stream>>>(L.N, b, L.cases, cellid, start, nl,
                                                     L.dscr);
  k_delta_grad<DIM, KER, KAHAN><<<g, bt, 0, L.stream>>>(L.N, b, L.cases, cellid, start, nl,
                                                        L.dscr);
  k_delta_rho<DIM, KER, KAHAN><<<g, bt, 0, L.stream>>>(L.N, b, L.cases, cellid, start, nl,
                                                       L.dscr, sph_gwbc, Rout, L.status);
  count_launch(L, 3);
}

template <int DIM, int KER, bool KAHAN>
void renorm_t(const LaunchCtx& L, Buffers b, const float4* Rin, float4* Rout, const int* cellid,
              const int* start, int sph_gwbc) {
  const int bt = kBlock;
  NList nl{L.nbr, L.nbr_cnt, L.kmax, L.vl, L.vcnt, L.kv, L.rref};
  k_renorm<DIM, KER, KAHAN><<<nblocks(L.N, bt), bt, 0, L.stream>>>(
      L.N, b, L.cases, cellid, start, nl, Rin, L.mask_self, sph_gwbc, Rout, L.status);
  count_launch(L);
}

// one instantiation per (dimension, kernel, Kahan) of the runtime configuration
template <template <int, int, bool> class Op, typename... A>
void dispatch(const LaunchCtx& L, A... a) {
  if (L.dim == 3) {
    if (L.kernel == SPH_KERNEL_QSK)
      L.kahan ? Op<3, 0, true>::run(L, a...) : Op<3, 0, false>::run(L, a...);
    else
      L.kahan ? Op<3, 1, true>::run(L, a...) : Op<3, 1, false>::run(L, a...);
  } else {
    if (L.kernel == SPH_KERNEL_QSK)
      L.kahan ? Op<2, 0, true>::run(L, a...) : Op<2, 0, false>::run(L, a...);
    else
      L.kahan ? Op<2, 1, true>::run(L, a...) : Op<2, 1, false>::run(L, a...);
  }
}

template <int DIM, int KER, bool KAHAN>
struct DeltaOp {
  static void run(const LaunchCtx& L, Buffers b, float4* Rout, const int* cellid,
                  const int* start, int sph_gwbc) {
    delta_t<DIM, KER, KAHAN>(L, b, Rout, cellid, start, sph_gwbc);
  }
};

template <int DIM, int KER, bool KAHAN>
struct RenormOp {
  static void run(const LaunchCtx& L, Buffers b, const float4* Rin, float4* Rout,
                  const int* cellid, const int* start, int sph_gwbc) {
    renorm_t<DIM, KER, KAHAN>(L, b, Rin, Rout, cellid, start, sph_gwbc);
  }
};

}  // namespace

void launch_delta_density(const LaunchCtx& L, Buffers b, float4* Rout, const int* cellid,
                          const int* start, int sph_gwbc) {
  dispatch<DeltaOp>(L, b, Rout, cellid, start, sph_gwbc);
}

void launch_renorm(const LaunchCtx& L, Buffers b, const float4* Rin, float4* Rout,
                   const int* cellid, const int* start, int sph_gwbc) {
  dispatch<RenormOp>(L, b, Rin, Rout, cellid, start, sph_gwbc);
}

}  // namespace sph
