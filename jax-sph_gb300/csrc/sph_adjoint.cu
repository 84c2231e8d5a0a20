// Hand-written reverse of one si_euler step for the differentiable form.
//
// Forward step (integrator.py:22-56, solver.py:705-949) on the path this
// reverse covers -- standard SPH with density summation, transport velocity
// (any tvf), optionally the generalized no-slip wall BC (solver.py:431-530)
// without gravity, bc_fn zeroing / prescribing wall velocities, no artificial
// viscosity; one case:
//   u' = u + dt a,  v' = u' + cv b,  x' = mod(x + dt v', L)        (kick-drift)
//   rho_k = m_k sum_l W(d_kl), p_k = P(rho_k)                       (fluid k)
//   walls w: S_w = sum_{j fluid} W_wj, ut_w = sum W_wj u'_j / (S_w + eps),
//            vt_w likewise, p_w = sum W_wj p_j / (S_w + eps),
//            rho_w = P^-1(p_w), u_w = 2 u'_w - ut_w, v_w = 2 v'_w - vt_w
//   a_k = sum_j T_kj B_kj,  b_k = sum_j T_kj pbg x_kj,  T_kj = K_kj h_kj,
//     K_kj = (V_k^2 + V_j^2)/m_k, V = m/rho, h = W'(d)/(d+eps), x_kj = x_k - x_j,
//     B_kj = -ps_kj x + 1/2 (rho_k u_k (w_k.x) + rho_j u_j (w_j.x)) + et_kj (u_k - u_j),
//     w = v - u, ps = (rho_j p_k + rho_k p_j)/(rho_k + rho_j),
//     et = 2 eta_k eta_j/(eta_k + eta_j + eps)
//   bc_fn: walls' a = b = 0 and u, v prescribed.
// With the neighbour list frozen (integer indices carry no gradient, as in
// the reference's jax.grad(..., allow_int=True)), the adjoints (la, lb) of the
// outputs a, b, (lr, lu) of x', u' map back in four passes over the recorded
// step (sorted order of that step; adjoint vectors in the original order):
//   A  per particle, over its pairs in both roles: the force's adjoints of
//      the pair inputs x, u, v, rho, p (F1..F3);
//   B  per wall: S_w, ut_w, vt_w and the wall pressure's adjoint
//      lp_w + lrho_w / P'(rho_w) (rho_w = P^-1(p_w));
//   C  per fluid particle: the Shepard sums of its wall neighbours passed on
//      to its u, v, p; the density adjoint mu = lrho + P'(rho) lp;
//   D  per particle: position adjoint (force, summation density with mu,
//      wall Shepard weights), then the kick-drift backwards.
// Pairs are used symmetrically; edges whose two directions differ only at
// exact cutoff ties carry W = W' = W'' = 0 there.
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
template <int DIM>
__device__ __forceinline__ void st3(float* a, long long o, const float3& v) {
  a[o * DIM] = v.x;
  a[o * DIM + 1] = v.y;
  if (DIM == 3) a[o * DIM + 2] = v.z;
}
__device__ __forceinline__ float dot(const float3& a, const float3& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
__device__ __forceinline__ float3 f3v(const float4& a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 operator+(const float3& a, const float3& b) {
  return make_float3(a.x + b.x, a.y + b.y, a.z + b.z);
}
__device__ __forceinline__ float3 operator-(const float3& a, const float3& b) {
  return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ float3 operator*(float s, const float3& a) {
  return make_float3(s * a.x, s * a.y, s * a.z);
}
__device__ __forceinline__ void acc(float3& a, const float3& b) {
  a.x += b.x;
  a.y += b.y;
  a.z += b.z;
}

// Lanes per particle of the reverse passes: S consecutive lanes of a warp
// share one particle, each summing every S-th of its pairs; the S partial
// sums are then added by a butterfly of shuffles (a fixed order: the result
// is the same on every run). Every lane of a warp takes part in the
// shuffles, so no lane leaves early.
__device__ __forceinline__ float group_sum(float v, int S) {
  for (int o = S >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float3 group_sum(float3 v, int S) {
  return make_float3(group_sum(v.x, S), group_sum(v.y, S), group_sum(v.z, S));
}

// The recorded forward data of one step.
struct Tape {
  const int* orig;
  const float4 *P4, *U4, *V4, *R4;
  const int* meta;
  const int *nbr, *cnt;
  int kmax;
};

// Per-step scratch of the reverse (sorted order of the recorded step).
struct Scratch {
  float4 *F1, *F2, *F3;  // force adjoints: (x, rho), (u, p), (v, -)
  float4 *WB, *WU, *WV;  // walls: (S + eps, lp_w, -, -), ut, vt
  float4 *GU, *GV;       // fluid: wall-borne u adjoint and mu, v adjoint
};

// One particle's quantities as the force pass used them.
struct Part {
  float3 x, u, v;
  float m, rho, p, eta;
  bool wall;
};
__device__ __forceinline__ Part load(const Tape& t, int k) {
  const float4 P = t.P4[k], U = t.U4[k], V = t.V4[k], R = t.R4[k];
  Part q;
  q.x = f3v(P);
  q.m = P.w;
  q.u = f3v(U);
  q.v = f3v(V);
  q.rho = R.x;
  q.p = R.y;
  q.eta = R.w;
  q.wall = is_wall(tag_of(t.meta[k]));
  return q;
}

// Minimum-image x_k - x_j, its length, W, h = W'/(d+eps) and dh/dd.
template <int DIM, int KER>
struct Geo {
  float3 x;
  float d, w, h, hd;
  __device__ __forceinline__ void eval(const float4& pk, const float4& pj, const CaseDev& c) {
    float d2;
    pair_dr<DIM>(pk, pj, c, x, d2);
    d = d2 > 0.f ? sqrtf(d2) : 0.f;
    const float inv = 1.f / (d + kEps);
    const float gw = kdw<KER>(d, c);
    w = kw<KER>(d, c);
    h = gw * inv;
    hd = kddw<KER>(d, c) * inv - gw * inv * inv;
  }
};

// Pass A: the force's adjoints of every particle's pair inputs, from its
// pairs as receiver (with its own la, lb) and as sender (with the
// neighbour's).
template <int DIM, int KER>
__global__ void __launch_bounds__(kBlock)
k_adj_force(long long N, Tape t, const CaseDev* cases, const float* __restrict__ la,
            const float* __restrict__ lb, Scratch s, unsigned* status, int S) {
  const long long gt = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long k0 = gt / S;
  const int sub = (int)(gt % S);
  const bool valid = k0 < N;
  const long long k = valid ? k0 : N - 1;  // idle lanes shadow the last particle
  const CaseDev& c = cases[0];
  const Part K = load(t, (int)k);
  const float4 pk = t.P4[k];
  const float3 zero = make_float3(0.f, 0.f, 0.f);
  const float3 lak = K.wall ? zero : ld3<DIM>(la, t.orig[k]);
  const float3 lbk = K.wall ? zero : ld3<DIM>(lb, t.orig[k]);
  const float Vk2 = (K.m / K.rho) * (K.m / K.rho);
  const float3 wk = K.v - K.u;
  const float pbg = c.p_bg_tvf;
  float3 gx = zero, gu = zero, gv = zero;
  float grho = 0.f, gp = 0.f;
  const int m = t.cnt[k];
  if (valid && sub == 0 && m > t.kmax) atomicOr(status, SPH_ERR_INVALID_ARG);
  const int mq = valid ? (m < t.kmax ? m : t.kmax) : 0;
  for (int q = sub; q < mq; q += S) {
    const int j = t.nbr[(long long)q * N + k];
    const Part J = load(t, j);
    Geo<DIM, KER> G;
    G.eval(pk, t.P4[j], c);
    const float3 laj = J.wall ? zero : ld3<DIM>(la, t.orig[j]);
    const float3 lbj = J.wall ? zero : ld3<DIM>(lb, t.orig[j]);
    const float Vj2 = (J.m / J.rho) * (J.m / J.rho);
    const float3 wj = J.v - J.u;
    const float rs = K.rho + J.rho;
    const float ps = (J.rho * K.p + K.rho * J.p) / rs;
    const float et = 2.f * K.eta * J.eta / (K.eta + J.eta + kEps);
    const float3 x = G.x;  // x_k - x_j
    const float wkx = dot(wk, x), wjx = dot(wj, x);
    // pair (k receives from j)
    {
      const float Kkj = (Vk2 + Vj2) / K.m;
      const float T = Kkj * G.h;
      const float3 B = (-ps) * x + (0.5f * K.rho * wkx) * K.u + (0.5f * J.rho * wjx) * J.u +
                       et * (K.u - J.u);
      const float sc = dot(lak, B) + pbg * dot(lbk, x);
      grho += sc * G.h * (-2.f * Vk2 / (K.rho * K.m));
      const float lau_k = dot(lak, K.u), lau_j = dot(lak, J.u);
      acc(gx, (sc * Kkj * G.hd / (G.d + kEps)) * x);
      acc(gx, T * (-ps) * lak + (T * 0.5f * K.rho * lau_k) * wk + (T * 0.5f * J.rho * lau_j) * wj +
                  (T * pbg) * lbk);
      const float lps = -T * dot(lak, x);
      gp += lps * J.rho / rs;
      grho += lps * (J.p - ps) / rs + T * 0.5f * lau_k * wkx;
      acc(gu, (T * 0.5f * K.rho * wkx + T * et) * lak - (T * 0.5f * K.rho * lau_k) * x);
      acc(gv, (T * 0.5f * K.rho * lau_k) * x);
    }
    // pair (j receives from k): x' = -x
    {
      const float Kjk = (Vj2 + Vk2) / J.m;
      const float T = Kjk * G.h;
      const float3 xp = (-1.f) * x;
      const float wkxp = -wkx, wjxp = -wjx;
      const float3 B = (-ps) * xp + (0.5f * J.rho * wjxp) * J.u + (0.5f * K.rho * wkxp) * K.u +
                       et * (J.u - K.u);
      const float sc = dot(laj, B) + pbg * dot(lbj, xp);
      grho += sc * G.h * (-2.f * Vk2 / (K.rho * J.m));
      const float lau_j = dot(laj, J.u), lau_k = dot(laj, K.u);
      // d x'/d x_k = -I
      acc(gx, (-sc * Kjk * G.hd / (G.d + kEps)) * xp);
      acc(gx, (-T) * ((-ps) * laj + (0.5f * J.rho * lau_j) * wj + (0.5f * K.rho * lau_k) * wk +
                      pbg * lbj));
      const float lps = -T * dot(laj, xp);
      gp += lps * J.rho / rs;
      grho += lps * (J.p - ps) / rs + T * 0.5f * lau_k * wkxp;
      acc(gu, (T * 0.5f * K.rho * wkxp - T * et) * laj - (T * 0.5f * K.rho * lau_k) * xp);
      acc(gv, (T * 0.5f * K.rho * lau_k) * xp);
    }
  }
  gx = group_sum(gx, S);
  gu = group_sum(gu, S);
  gv = group_sum(gv, S);
  grho = group_sum(grho, S);
  gp = group_sum(gp, S);
  if (!valid || sub != 0) return;
  s.F1[k] = make_float4(gx.x, gx.y, gx.z, grho);
  s.F2[k] = make_float4(gu.x, gu.y, gu.z, gp);
  s.F3[k] = make_float4(gv.x, gv.y, gv.z, 0.f);
}

// Pass B: the walls' Shepard sums and wall-pressure adjoint.
template <int DIM, int KER>
__global__ void __launch_bounds__(kBlock)
k_adj_wall(long long N, Tape t, const CaseDev* cases, Scratch s, int S) {
  const long long gt = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long k0 = gt / S;
  const int sub = (int)(gt % S);
  const long long k = k0 < N ? k0 : N - 1;
  const bool valid = k0 < N && is_wall(tag_of(t.meta[k]));  // uniform over the S lanes
  const CaseDev& c = cases[0];
  const float4 pk = t.P4[k];
  float Sw = 0.f;
  float3 su = make_float3(0.f, 0.f, 0.f), sv = su;
  const int m = t.cnt[k];
  const int mq = valid ? (m < t.kmax ? m : t.kmax) : 0;
  for (int q = sub; q < mq; q += S) {
    const int j = t.nbr[(long long)q * N + k];
    if (tag_of(t.meta[j]) != FLUID) continue;
    Geo<DIM, KER> G;
    G.eval(pk, t.P4[j], c);
    Sw += G.w;
    acc(su, G.w * f3v(t.U4[j]));
    acc(sv, G.w * f3v(t.V4[j]));
  }
  Sw = group_sum(Sw, S);
  su = group_sum(su, S);
  sv = group_sum(sv, S);
  if (!valid || sub != 0) return;
  const float den = Sw + kEps;
  const float4 F1 = s.F1[k], F2 = s.F2[k];
  const float lp = F2.w + F1.w / eos_dp(t.R4[k].x, c);  // rho_w = P^-1(p_w)
  s.WB[k] = make_float4(den, lp, 0.f, 0.f);
  s.WU[k] = make_float4(su.x / den, su.y / den, su.z / den, 0.f);
  s.WV[k] = make_float4(sv.x / den, sv.y / den, sv.z / den, 0.f);
}

// Pass C: what the walls' Shepard sums pass on to each fluid particle's u,
// v and p, and its density adjoint mu.
template <int DIM, int KER>
__global__ void __launch_bounds__(kBlock)
k_adj_mu(long long N, Tape t, const CaseDev* cases, Scratch s, int walls, int S) {
  const long long gt = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long k0 = gt / S;
  const int sub = (int)(gt % S);
  const long long k = k0 < N ? k0 : N - 1;
  const bool valid = k0 < N;
  const float3 zero = make_float3(0.f, 0.f, 0.f);
  const bool wall = is_wall(tag_of(t.meta[k]));  // uniform over the S lanes
  const CaseDev& c = cases[0];
  float3 gu = zero, gv = zero;
  float gp = 0.f;
  if (walls) {
    const float4 pk = t.P4[k];
    const int m = t.cnt[k];
    const int mq = (valid && !wall) ? (m < t.kmax ? m : t.kmax) : 0;
    for (int q = sub; q < mq; q += S) {
      const int j = t.nbr[(long long)q * N + k];
      if (!is_wall(tag_of(t.meta[j]))) continue;
      Geo<DIM, KER> G;
      G.eval(t.P4[j], pk, c);
      const float4 WB = s.WB[j];
      const float cw = G.w / WB.x;
      // u_w = 2 u'_w - ut_w: the adjoint of ut_w is minus that of u_w
      acc(gu, (-cw) * f3v(s.F2[j]));
      acc(gv, (-cw) * f3v(s.F3[j]));
      gp += cw * WB.y;
    }
    gu = group_sum(gu, S);
    gv = group_sum(gv, S);
    gp = group_sum(gp, S);
  }
  if (!valid || sub != 0) return;
  if (wall) {
    s.GU[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    s.GV[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const float4 F1 = s.F1[k], F2 = s.F2[k];
  const float mu = F1.w + eos_dp(t.R4[k].x, c) * (F2.w + gp);
  s.GU[k] = make_float4(gu.x, gu.y, gu.z, mu);
  s.GV[k] = make_float4(gv.x, gv.y, gv.z, 0.f);
}

// Pass D: position adjoints and the kick-drift backwards (lr, lu in place;
// la, lb of the step's inputs into la_out, lb_out).
template <int DIM, int KER>
__global__ void __launch_bounds__(kBlock)
k_adj_grad(long long N, Tape t, const CaseDev* cases, Scratch s, float* lr, float* lu,
           float* la_out, float* lb_out, int S) {
  const long long gt = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long k0 = gt / S;
  const int sub = (int)(gt % S);
  const bool valid = k0 < N;
  const long long k = valid ? k0 : N - 1;
  const CaseDev& c = cases[0];
  const float3 zero = make_float3(0.f, 0.f, 0.f);
  const Part K = load(t, (int)k);
  const float4 pk = t.P4[k];
  const float mu_k = K.wall ? 0.f : s.GU[k].w;
  float3 gx = zero;
  // the wall's own Shepard terms (k a wall): adjoints of ut, vt, p_w
  float4 WBk = make_float4(1.f, 0.f, 0.f, 0.f);
  float3 lut = zero, lvt = zero, ut = zero, vt = zero;
  if (K.wall) {
    WBk = s.WB[k];
    lut = (-1.f) * f3v(s.F2[k]);
    lvt = (-1.f) * f3v(s.F3[k]);
    ut = f3v(s.WU[k]);
    vt = f3v(s.WV[k]);
  }
  const int m = t.cnt[k];
  const int mq = valid ? (m < t.kmax ? m : t.kmax) : 0;
  for (int q = sub; q < mq; q += S) {
    const int j = t.nbr[(long long)q * N + k];
    const Part J = load(t, j);
    Geo<DIM, KER> G;
    G.eval(pk, t.P4[j], c);
    // summation density (fluid receivers), both directions
    const float mu_j = J.wall ? 0.f : s.GU[j].w;
    acc(gx, (G.h * (mu_k * K.m + mu_j * J.m)) * G.x);
    if (K.wall && !J.wall) {
      // dW_kj/dx_k = h x_kj, weight of j in the wall's Shepard sums
      const float cs = (dot(lut, J.u - ut) + dot(lvt, J.v - vt) + WBk.y * (J.p - K.p)) / WBk.x;
      acc(gx, (cs * G.h) * G.x);
    } else if (!K.wall && J.wall) {
      const float4 WB = s.WB[j];
      const float3 lutj = (-1.f) * f3v(s.F2[j]), lvtj = (-1.f) * f3v(s.F3[j]);
      const float cs = (dot(lutj, K.u - f3v(s.WU[j])) + dot(lvtj, K.v - f3v(s.WV[j])) +
                        WB.y * (K.p - J.p)) /
                       WB.x;
      // the pair (j, k) seen from the wall: x_jk = -x_kj, and x_k enters with -I
      acc(gx, (cs * G.h) * G.x);
    }
  }
  gx = group_sum(gx, S) + f3v(s.F1[k]);
  if (!valid || sub != 0) return;
  const long long ok = t.orig[k];
  const float3 lx = ld3<DIM>(lr, ok) + gx;
  if (K.wall) {
    // the walls' velocities and rates are prescribed by bc_fn
    st3<DIM>(lr, ok, lx);
    st3<DIM>(lu, ok, zero);
    st3<DIM>(la_out, ok, zero);
    st3<DIM>(lb_out, ok, zero);
    return;
  }
  float3 lv = f3v(s.F3[k]) + f3v(s.GV[k]);
  float3 lvel = ld3<DIM>(lu, ok) + f3v(s.F2[k]) + f3v(s.GU[k]);
  lv = lv + c.dt * lx;       // x' = x + dt v'
  lvel = lvel + lv;          // v' = u' + cv b
  st3<DIM>(lr, ok, lx);
  st3<DIM>(lu, ok, lvel);     // u' = u + dt a
  st3<DIM>(la_out, ok, c.dt * lvel);
  st3<DIM>(lb_out, ok, c.cv * lv);
}

// The tape slot of the step just taken, one thread per particle (the
// neighbour list row by row, coalesced), its senders as 32-bit sorted
// indices whatever the passes' list format: FMT 0 32-bit rows (generic
// passes), 1 words of four 16-bit offsets j - i modulo N, 2 words of four
// 32-bit indices (the lean passes).
template <int FMT>
__device__ __forceinline__ int list_sender(const int* nbr, long long N, long long k, int q) {
  if (FMT == 0) return nbr[(long long)q * N + k];
  if (FMT == 1) {
    const uint2 w = reinterpret_cast<const uint2*>(nbr)[(long long)(q >> 2) * N + k];
    const unsigned h = (q & 2) ? w.y : w.x;
    long long j = k + (int)(short)(unsigned short)(h >> ((q & 1) * 16));
    j += j < 0 ? N : 0;
    j -= j >= N ? N : 0;
    return (int)j;
  }
  const int4 w = reinterpret_cast<const int4*>(nbr)[(long long)(q >> 2) * N + k];
  const int r = q & 3;
  return r == 0 ? w.x : (r == 1 ? w.y : (r == 2 ? w.z : w.w));
}

template <int FMT>
__global__ void k_tape_record(long long N, Buffers b, const float4* R4, const int* nbr,
                              const int* cnt, int kmax, int* t_orig, float4* t_P4, float4* t_U4,
                              float4* t_V4, float4* t_R4, int* t_meta, int* t_nbr, int* t_cnt) {
  const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k >= N) return;
  t_orig[k] = b.ORIG[k];
  t_P4[k] = b.P4[k];
  t_U4[k] = b.U4[k];
  t_V4[k] = b.V4[k];
  t_R4[k] = R4[k];
  t_meta[k] = b.META[k];
  const int m = cnt[k];
  t_cnt[k] = m;
  const int e = m < kmax ? m : kmax;
  for (int q = 0; q < e; ++q) t_nbr[(long long)q * N + k] = list_sender<FMT>(nbr, N, k, q);
}

// Lanes per particle of the reverse passes (1, 2, 4 or 8): as many as keep
// about two full waves of 256-thread blocks on the device, so that a small
// case (the differentiable form's 16,384 particles) still fills every SM.
inline int adj_lanes(long long n) {
  int sms = 0, dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
    return 1;
  const long long target = 2LL * sms * 2048;  // threads
  int S = 1;
  while (S < 8 && n * (2 * S) <= target) S *= 2;
  return S;
}

template <int DIM, int KER>
void adjoint_t(const LaunchCtx& L, const Tape& t, const Scratch& s, const float* la,
               const float* lb, float* la_out, float* lb_out, float* lr, float* lu,
               int walls) {
  const int S = adj_lanes(L.N);
  const long long threads = L.N * S;
  const int g = (int)((threads + kBlock - 1) / kBlock);
  k_adj_force<DIM, KER><<<g, kBlock, 0, L.stream>>>(L.N, t, L.cases, la, lb, s, L.status, S);
  if (walls) k_adj_wall<DIM, KER><<<g, kBlock, 0, L.stream>>>(L.N, t, L.cases, s, S);
  k_adj_mu<DIM, KER><<<g, kBlock, 0, L.stream>>>(L.N, t, L.cases, s, walls, S);
  k_adj_grad<DIM, KER><<<g, kBlock, 0, L.stream>>>(L.N, t, L.cases, s, lr, lu, la_out, lb_out,
                                                    S);
}

}  // namespace

void launch_tape_record(const LaunchCtx& L, Buffers b, const float4* R4, int* t_orig,
                        float4* t_P4, float4* t_U4, float4* t_V4, float4* t_R4, int* t_meta,
                        int* t_nbr, int* t_cnt) {
  const int g = (int)((L.N + kBlock - 1) / kBlock);
#define SPH_TAPE(F)                                                                          \
  k_tape_record<F><<<g, kBlock, 0, L.stream>>>(L.N, b, R4, L.nbr, L.nbr_cnt, L.kmax, t_orig,  \
                                               t_P4, t_U4, t_V4, t_R4, t_meta, t_nbr, t_cnt)
  if (L.lean == 1) SPH_TAPE(1);
  else if (L.lean == 2) SPH_TAPE(2);
  else SPH_TAPE(0);
#undef SPH_TAPE
}

void launch_adjoint(const LaunchCtx& L, const AdjTape& at, const AdjScratch& as, const float* la,
                    const float* lb, float* la_out, float* lb_out, float* lr, float* lu,
                    int walls) {
  Tape t{at.orig, at.P4, at.U4, at.V4, at.R4, at.meta, at.nbr, at.cnt, L.kmax};
  Scratch s{as.F1, as.F2, as.F3, as.WB, as.WU, as.WV, as.GU, as.GV};
  if (L.dim == 3) {
    if (L.kernel == SPH_KERNEL_QSK) adjoint_t<3, 0>(L, t, s, la, lb, la_out, lb_out, lr, lu, walls);
    else adjoint_t<3, 1>(L, t, s, la, lb, la_out, lb_out, lr, lu, walls);
  } else {
    if (L.kernel == SPH_KERNEL_QSK) adjoint_t<2, 0>(L, t, s, la, lb, la_out, lb_out, lr, lu, walls);
    else adjoint_t<2, 1>(L, t, s, la, lb, la_out, lb_out, lr, lu, walls);
  }
}

}  // namespace sph
