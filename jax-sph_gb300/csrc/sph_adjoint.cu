// Hand-written reverse of one si_euler step for the differentiable form.
//
// Forward step (integrator.py:22-56, solver.py:705-949) on the path this
// reverse covers -- standard SPH, density summation, tvf = 0, periodic box,
// fluid only, no artificial viscosity:
//   u' = u + dt a,  r' = mod(r + dt u', L)
//   rho_k = m_k sum_l W(d_kl),  p_k = P(rho_k)
//   a'_k  = sum_j K_kj h_kj B_kj,  K_kj = (m_k^2/rho_k^2 + m_j^2/rho_j^2)/m_k,
//           h = W'(d)/(d+eps),  B_kj = -ps_kj x_kj + et_kj (u'_k - u'_j),
//           ps = (rho_j p_k + rho_k p_j)/(rho_k + rho_j),
//           et = 2 eta_k eta_j/(eta_k + eta_j + eps),  x_kj = r'_k - r'_j
// (the transport-velocity stress vanishes with v = u and contributes no
// derivative because v and u move together). With the neighbour list frozen
// (integer indices carry no gradient, as in the reference's
// jax.grad(..., allow_int=True)), given the adjoints la of a', lr of r' and
// lu of u' the reverse is
//   mu_k  = sum_j h [dKa B.la_k - K_kj D_k x.la_k - dKb B.la_j + K_jk D_k x.la_j]
//   lr'_k = lr_k + sum_j [K_kj(-ps h la_k + h' (B.la_k) x/(d+eps))
//                         + K_jk(ps h la_j - h' (B.la_j) x/(d+eps))
//                         + h x (mu_k m_k + mu_j m_j)]
//   lu'_k = lu_k + sum_j h et (K_kj la_k - K_jk la_j) + dt lr'_k
//   outputs: lr = lr'_k, lu = lu'_k, la = dt lu'_k
// with dKa = dK_kj/drho_k = -2 m_k/rho_k^3, dKb = dK_jk/drho_k =
// -2 m_k^2/(rho_k^3 m_j), D_k = dps/drho_k = (rho_j P'(rho_k) + p_j - ps) /
// (rho_k + rho_j). Pairs are used symmetrically; edges whose two directions
// differ only at exact cutoff ties carry W = W' = W'' = 0 there.
//
// Each recorded step keeps the sorted order, positions, velocities, density,
// pressure and neighbour list of its forward pass ("tape slot"); the adjoint
// vectors live in the original particle order.
#include "sph_internal.cuh"

namespace sph {

namespace {

constexpr int kBlock = 256;

// d2W/dr2 of the kernels (kernel.py:51-103 differentiated twice).
template <int KER>
__device__ __forceinline__ float kddw(float r, const CaseDev& c) {
  const float q = r * c.inv_h;
  if (KER == 0) {
    const float q1 = fmaxf(0.f, 1.f - q), q2 = fmaxf(0.f, 2.f - q), q3 = fmaxf(0.f, 3.f - q);
    // d/dr [dsigma (q3^4 - 6 q2^4 + 15 q1^4)] = dsigma * (-4/h) (q3^3 - 6 q2^3 + 15 q1^3)
    return -4.f * c.dsigma * c.inv_h *
           (q3 * q3 * q3 - 6.f * q2 * q2 * q2 + 15.f * q1 * q1 * q1);
  } else {
    const float q1 = fmaxf(0.f, 1.f - 0.5f * q);
    // d/dr [dsigma q q1^3] = dsigma/h (q1^3 - 1.5 q q1^2)
    return c.dsigma * c.inv_h * (q1 * q1 * q1 - 1.5f * q * q1 * q1);
  }
}

__device__ __forceinline__ float eos_dp(float rho, const CaseDev& c) {
  if (c.eos == SPH_EOS_TAIT) {
    if (c.gamma == 1.0f) return c.p_ref / c.rho_ref;
    return c.p_ref * c.gamma * powf(rho / c.rho_ref, c.gamma - 1.f) / c.rho_ref;
  }
  return c.rie_k;
}

template <int DIM>
__device__ __forceinline__ float3 ld3(const float* a, long long o) {
  return make_float3(a[o * DIM], a[o * DIM + 1], DIM == 3 ? a[o * DIM + 2] : 0.f);
}
__device__ __forceinline__ float dot(const float3& a, const float3& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}

// Pair quantities shared by the two passes.
template <int DIM, int KER>
struct Pair {
  float3 x;     // r'_k - r'_j (minimum image)
  float inv, h, hp, K_kj, K_jk, ps, et, Dk;
  float3 B;     // B_kj
  __device__ __forceinline__ void eval(const float4& rk, const float4& rj, float rho_k,
                                       float rho_j, float p_k, float p_j, float eta_k,
                                       float eta_j, const float3& uk, const float3& uj,
                                       const CaseDev& c) {
    float d2;
    pair_dr<DIM>(rk, rj, c, x, d2);
    const float d = d2 > 0.f ? sqrtf(d2) : 0.f;
    inv = 1.f / (d + kEps);
    const float gw = kdw<KER>(d, c);
    h = gw * inv;
    hp = kddw<KER>(d, c) * inv - gw * inv * inv;
    const float mk = rk.w, mj = rj.w;
    const float vk = mk / rho_k, vj = mj / rho_j;
    K_kj = (vk * vk + vj * vj) / mk;
    K_jk = (vk * vk + vj * vj) / mj;
    ps = (rho_j * p_k + rho_k * p_j) / (rho_k + rho_j);
    et = 2.f * eta_k * eta_j / (eta_k + eta_j + kEps);
    Dk = (rho_j * eos_dp(rho_k, c) + p_j - ps) / (rho_k + rho_j);
    B = make_float3(-ps * x.x + et * (uk.x - uj.x), -ps * x.y + et * (uk.y - uj.y),
                    -ps * x.z + et * (uk.z - uj.z));
  }
};

struct Tape {
  const int* orig;
  const float4 *P4, *U4, *R4;
  const int *nbr, *cnt;
  int kmax;
};

// Pass 1: density adjoint mu_k (sorted order of the recorded step).
template <int DIM, int KER>
__global__ void __launch_bounds__(kBlock)
k_adj_mu(long long N, Tape t, const CaseDev* cases, const float* __restrict__ la, float* mu,
         unsigned* status) {
  long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k >= N) return;
  const CaseDev& c = cases[0];
  const float4 rk = t.P4[k], Uk = t.U4[k], Rk = t.R4[k];
  const float3 uk = make_float3(Uk.x, Uk.y, Uk.z);
  const float rho_k = Rk.x, p_k = Rk.y, eta_k = Rk.w, mk = rk.w;
  const float3 lak = ld3<DIM>(la, t.orig[k]);
  const float dKa = -2.f * mk / (rho_k * rho_k * rho_k);
  const int m = t.cnt[k];
  if (m > t.kmax) atomicOr(status, SPH_ERR_INVALID_ARG);
  float acc = 0.f;
  for (int q = 0; q < m && q < t.kmax; ++q) {
    const int j = t.nbr[(long long)q * N + k];
    const float4 rj = t.P4[j], Uj = t.U4[j], Rj = t.R4[j];
    Pair<DIM, KER> P;
    P.eval(rk, rj, rho_k, Rj.x, p_k, Rj.y, eta_k, Rj.w, uk, make_float3(Uj.x, Uj.y, Uj.z), c);
    const float3 laj = ld3<DIM>(la, t.orig[j]);
    const float dKb = -2.f * mk * mk / (rho_k * rho_k * rho_k * rj.w);
    acc += P.h * (dKa * dot(P.B, lak) - P.K_kj * P.Dk * dot(P.x, lak) - dKb * dot(P.B, laj) +
                  P.K_jk * P.Dk * dot(P.x, laj));
  }
  mu[k] = acc;
}

// Pass 2: adjoints of r, u and a before the step (original order).
template <int DIM, int KER>
__global__ void __launch_bounds__(kBlock)
k_adj_grad(long long N, Tape t, const CaseDev* cases, const float* __restrict__ la_in,
           const float* __restrict__ mu, float* lr, float* lu, float* la_out) {
  long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k >= N) return;
  const CaseDev& c = cases[0];
  const float4 rk = t.P4[k], Uk = t.U4[k], Rk = t.R4[k];
  const float3 uk = make_float3(Uk.x, Uk.y, Uk.z);
  const float rho_k = Rk.x, p_k = Rk.y, eta_k = Rk.w, mk = rk.w;
  const long long ok = t.orig[k];
  const float3 lak = ld3<DIM>(la_in, ok);
  const float muk_mk = mu[k] * mk;
  float3 gr = make_float3(0.f, 0.f, 0.f), gu = make_float3(0.f, 0.f, 0.f);
  const int m = t.cnt[k];
  for (int q = 0; q < m && q < t.kmax; ++q) {
    const int j = t.nbr[(long long)q * N + k];
    const float4 rj = t.P4[j], Uj = t.U4[j], Rj = t.R4[j];
    Pair<DIM, KER> P;
    P.eval(rk, rj, rho_k, Rj.x, p_k, Rj.y, eta_k, Rj.w, uk, make_float3(Uj.x, Uj.y, Uj.z), c);
    const float3 laj = ld3<DIM>(la_in, t.orig[j]);
    const float bk = dot(P.B, lak), bj = dot(P.B, laj);
    const float sx = P.hp * P.inv * (P.K_kj * bk - P.K_jk * bj) + P.h * (muk_mk + mu[j] * rj.w);
    const float sl = P.ps * P.h;
    gr.x += -P.K_kj * sl * lak.x + P.K_jk * sl * laj.x + sx * P.x.x;
    gr.y += -P.K_kj * sl * lak.y + P.K_jk * sl * laj.y + sx * P.x.y;
    gr.z += -P.K_kj * sl * lak.z + P.K_jk * sl * laj.z + sx * P.x.z;
    const float he = P.h * P.et;
    gu.x += he * (P.K_kj * lak.x - P.K_jk * laj.x);
    gu.y += he * (P.K_kj * lak.y - P.K_jk * laj.y);
    gu.z += he * (P.K_kj * lak.z - P.K_jk * laj.z);
  }
  const float3 lrk = ld3<DIM>(lr, ok), luk = ld3<DIM>(lu, ok);
  const float3 r_tot = make_float3(lrk.x + gr.x, lrk.y + gr.y, lrk.z + gr.z);
  const float3 u_tot = make_float3(luk.x + gu.x + c.dt * r_tot.x, luk.y + gu.y + c.dt * r_tot.y,
                                   luk.z + gu.z + c.dt * r_tot.z);
  lr[ok * DIM] = r_tot.x;
  lr[ok * DIM + 1] = r_tot.y;
  lu[ok * DIM] = u_tot.x;
  lu[ok * DIM + 1] = u_tot.y;
  la_out[ok * DIM] = c.dt * u_tot.x;
  la_out[ok * DIM + 1] = c.dt * u_tot.y;
  if (DIM == 3) {
    lr[ok * DIM + 2] = r_tot.z;
    lu[ok * DIM + 2] = u_tot.z;
    la_out[ok * DIM + 2] = c.dt * u_tot.z;
  }
}

template <int DIM, int KER>
void adjoint_t(const LaunchCtx& L, const Tape& t, float* mu, const float* la_in, float* la_out,
               float* lr, float* lu) {
  const int g = (int)((L.N + kBlock - 1) / kBlock);
  k_adj_mu<DIM, KER><<<g, kBlock, 0, L.stream>>>(L.N, t, L.cases, la_in, mu, L.status);
  k_adj_grad<DIM, KER><<<g, kBlock, 0, L.stream>>>(L.N, t, L.cases, la_in, mu, lr, lu, la_out);
}

// The tape slot of the step just taken, one thread per particle (the
// neighbour list row by row, coalesced).
__global__ void k_tape_record(long long N, Buffers b, const float4* R4, const int* nbr,
                              const int* cnt, int kmax, int* t_orig, float4* t_P4, float4* t_U4,
                              float4* t_R4, int* t_nbr, int* t_cnt) {
  const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k >= N) return;
  t_orig[k] = b.ORIG[k];
  t_P4[k] = b.P4[k];
  t_U4[k] = b.U4[k];
  t_R4[k] = R4[k];
  const int m = cnt[k];
  t_cnt[k] = m;
  const int e = m < kmax ? m : kmax;
  for (int q = 0; q < e; ++q) t_nbr[(long long)q * N + k] = nbr[(long long)q * N + k];
}

}  // namespace

void launch_tape_record(const LaunchCtx& L, Buffers b, const float4* R4, int* t_orig,
                        float4* t_P4, float4* t_U4, float4* t_R4, int* t_nbr, int* t_cnt) {
  const int g = (int)((L.N + kBlock - 1) / kBlock);
  k_tape_record<<<g, kBlock, 0, L.stream>>>(L.N, b, R4, L.nbr, L.nbr_cnt, L.kmax, t_orig, t_P4,
                                            t_U4, t_R4, t_nbr, t_cnt);
}

void launch_adjoint(const LaunchCtx& L, const int* orig, const float4* P4, const float4* U4,
                    const float4* R4, const int* nbr, const int* cnt, float* mu,
                    const float* la_in, float* la_out, float* lr, float* lu) {
  Tape t{orig, P4, U4, R4, nbr, cnt, L.kmax};
  if (L.dim == 3) {
    if (L.kernel == SPH_KERNEL_QSK) adjoint_t<3, 0>(L, t, mu, la_in, la_out, lr, lu);
    else adjoint_t<3, 1>(L, t, mu, la_in, la_out, lr, lu);
  } else {
    if (L.kernel == SPH_KERNEL_QSK) adjoint_t<2, 0>(L, t, mu, la_in, la_out, lr, lu);
    else adjoint_t<2, 1>(L, t, mu, la_in, la_out, lr, lu);
  }
}

}  // namespace sph
