// Internal declarations of the GB300 jax-sph hot path (not part of the ABI).
//
// Device layout (particles always kept in cell-sorted order after a binning):
//   P4  float4  (x, y, z, m)          positions + mass
//   U4  float4  (u.xyz, rho_state)    velocity + state density
//   V4  float4  (v.xyz, p_state)      transport velocity + state pressure
//   A4  float4  (dudt.xyz, drhodt)    accelerations + density rate
//   A2  float4  (dvdt.xyz, -)         transport acceleration
//   ETA float, META int (case << 4 | tag), ORIG int (original index)
//   NW4 float4  wall normals (Riemann/free-slip only)
//   R4  float4  (rho_new, p_new, drhodt_new, -) produced by the density pass
//   UT4 float4  Shepard-averaged wall velocity (Riemann + wall BC)
// Every pass writes only arrays that no concurrent thread of the same pass
// reads, so no pass needs a grid-wide barrier.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <climits>

#include <string>

#include "../../include/sph_gb300.h"

namespace sph {

constexpr float kEps = 2.220446049250313e-16f;  // jnp.finfo(float).eps, solver.py:21
constexpr int kTagBits = 4;
constexpr int kTagMask = 0xF;

enum Tag { FLUID = 0, SOLID_WALL = 1, MOVING_WALL = 2, DIRICHLET_WALL = 3 };
// Padding particles (Tag.PAD_VALUE = -1 in the state): binned into a cell of
// their own past the case's grid that no walk visits, with no lists.
constexpr int PAD = 15;

// Neighbour-list slots per particle. The density pass stages them in shared
// memory (kListSlots * 256 threads * 4 B = 40 KB per block); a particle with
// more neighbours makes the passes walk its cells instead.
constexpr int kListSlots = 40;

// Verlet candidate slots per particle: sized per handle from the expected
// candidate count (the volume of the Verlet sphere over dx^d, times 1.5, plus
// 8), between these bounds; a particle with more walks its cells instead.
constexpr int kVerletMinSlots = 32;
constexpr int kVerletMaxSlots = 384;
// Threads per block of the candidate-list build for kv slots (its shared
// memory, 8 kv bytes per thread, stays under 100 KB).
inline int verlet_block(int kv) { return kv <= 96 ? 128 : (kv <= 192 ? 64 : 32); }

// Per-case constants, all rounded to float32 the way the reference's
// float32 program sees them.
//
// The particles are binned into cells of the reference's cell size divided by
// sub (1 or 2) along each axis. With sub = 2 the fine size is exactly half the
// reference's (a power-of-two split), so fl(r / (s/2)) = 2 fl(r / s) and the
// reference's cell index is the fine index >> 1: the reference's cell
// occupancy is the sum over its 2^d fine cells.
struct CaseDev {
  float box[3], half[3];
  float cell_size[3];  // binned (fine) cell size
  int nc[3];          // fine cells per side (1 along an axis with fewer than 3 reference cells)
  int sub[3];         // fine cells per reference cell along each axis
  int rad[3];         // cells walked on each side of the receiver's cell (0: whole axis)
  int mult[3];        // hash multipliers (1, nx, nx*ny)
  int use_cells;      // reference builds a cell list (cells >= 3 on every axis)
  int cell_off, ncell;
  int p_off, n;
  int cell_cap;       // cell capacity for the CELL_LIST_OVERFLOW test
  long long edge_cap; // neighbour-list capacity for NEIGHBOR_LIST_OVERFLOW
  float cutoff_sq;
  float inv_h, sigma, dsigma;  // W(r) = sigma*f(q); dW/dr = dsigma*g(q)
  float dt, cv;       // f32(dt), f32(tvf*0.5*dt) of si_euler
  float dt_rho;       // WCSPH dt of density evolution
  int eos;
  float p_ref, rho_ref, p_bg, gamma, inv_gamma, rie_k;  // rie_k = 100*u_ref^2
  float p_bg_tvf;     // eos.p_fn(0)
  float c_ref, eta_limiter;
  float av_alpha, av_hab, av_cab, av_eps;
  float delta_coef;   // diff_alpha * h * c_ref * rho_ref (DELTA diffusive acceleration)
  float delta_rho_coef;  // c_ref * diff_delta * h (DELTA density diffusion)
  int g_kind;
  float g[3], g_lo, g_hi;
  int bc_kind;
  float u_lid[3];
  float bc_T[2], bc_x[2];  // SPH_BC_HT temperatures and inflow / outflow bounds
  // Fast membership test (every axis has >= 5 cells, so adjacent-cell images
  // are minimum images): squared distances below cut_lo are edges, above
  // cut_hi are not, and only the band between takes the reference metric.
  int fast;
  float cut_lo, cut_hi;
  float inv_box[3];
  // Row trimming of the walk (fast cases): a (y, z) row of cells is skipped
  // when its nearest point is farther than sqrt(trim_r2), and its x extent is
  // cut to the chord of that sphere; trim_m (64 ulp of the largest side)
  // absorbs every rounding of the bounds and of the hash.
  float trim_r2, trim_m;
  float inv_cs[3];
  // Verlet candidate list: the senders within sqrt(v_r2) of the receiver at
  // the last rebuild, found by walking vrad cells on each side; a rebuild is
  // due once some particle has moved farther than sqrt(v_dmax2) since (half
  // the skin, less rounding margins), so every sender within the cutoff stays
  // in the list until then. Without a skin v_dmax2 = 0: any motion rebuilds.
  int vrad[3];
  float v_r2, v_dmax2;
  int cref_off, ncref;  // this case's reference cells in the per-step occupancy count
  double dt64, box64[3];  // float64 drift of the precision form
  // matscipy backend: float64 minimum-image distance < cutoff (kept last: the
  // hot loops read the fields above)
  double cut64_sq, mat_box[3];
  int f64_metric;
};

struct Buffers {
  float4 *P4, *U4, *V4, *A4, *A2, *NW4;
  float* ETA;
  int *META, *ORIG;
  double4_32a* RD;  // float64 positions of the precision form (else null)
  float4* TH4;      // heat conduction: (T, dTdt, kappa, Cp) (else null)
  float2* TO;       // heat conduction: the forward pass's new (T, dTdt), in the
                    // order of the buffers it ran on (shared by both sets, like R4)
};

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ int tag_of(int meta) { return meta & kTagMask; }
__device__ __forceinline__ int case_of(int meta) { return meta >> kTagBits; }
__device__ __forceinline__ bool is_wall(int tag) { return tag >= 1 && tag <= 3; }

// jnp.mod(x, L) for L > 0: fmod then add L to a negative non-zero remainder.
// For -L < x < 2L the fmod is x or x - L, both exact (Sterbenz), so the fast
// branch equals fmodf bit for bit; other inputs take fmodf itself.
__device__ __forceinline__ float jmod(float x, float L) {
  if (x >= L) {
    if (x < 2.0f * L) return __fsub_rn(x, L);
  } else if (x >= 0.0f || x != x) {
    return x;
  } else if (x > -L) {
    return __fadd_rn(x, L);
  }
  float t = fmodf(x, L);
  if (t != 0.0f && t < 0.0f) t = __fadd_rn(t, L);
  return t;
}

// periodic_displacement (jax_md/space.py:170-181), component-wise, no FMA.
__device__ __forceinline__ float pdisp(float d, float L, float half) {
  return __fsub_rn(jmod(__fadd_rn(d, half), L), half);
}

template <int DIM>
__device__ __forceinline__ float3 pdisp3(const float4& a, const float4& b, const CaseDev& c) {
  float3 r;
  r.x = pdisp(__fsub_rn(a.x, b.x), c.box[0], c.half[0]);
  r.y = pdisp(__fsub_rn(a.y, b.y), c.box[1], c.half[1]);
  r.z = (DIM == 3) ? pdisp(__fsub_rn(a.z, b.z), c.box[2], c.half[2]) : 0.0f;
  return r;
}

// square_distance summed left to right without contraction (space.py:184-192).
template <int DIM>
__device__ __forceinline__ float sqd(const float3& d) {
  float s = __fadd_rn(__fmul_rn(d.x, d.x), __fmul_rn(d.y, d.y));
  if (DIM == 3) s = __fadd_rn(s, __fmul_rn(d.z, d.z));
  return s;
}

// Neighbour-list membership of edge (receiver a, sender b): the reference
// prunes with metric(r[sender], r[receiver]) < cutoff_sq (partition.py:897).
// The matscipy backend's membership: the pair's distance in float64 from
// the float32 positions, nearest periodic image, strictly below the cutoff.
template <int DIM>
__device__ __forceinline__ bool is_edge_f64(const float4& recv, const float4& send,
                                            const CaseDev& c) {
  const double p[3] = {(double)send.x - (double)recv.x, (double)send.y - (double)recv.y,
                       DIM == 3 ? (double)send.z - (double)recv.z : 0.0};
  double s = 0.0;
  for (int d = 0; d < DIM; ++d) {
    const double x = p[d] - c.mat_box[d] * rint(p[d] / c.mat_box[d]);
    s += x * x;
  }
  return s < c.cut64_sq;
}

// The jax_md membership (float32 reference metric).
template <int DIM>
__device__ __forceinline__ bool is_edge(const float4& recv, const float4& send, const CaseDev& c) {
  return sqd<DIM>(pdisp3<DIM>(send, recv, c)) < c.cutoff_sq;
}

// Kernel value and radial derivative (kernel.py:51-103). KER 0 = quintic, 1 = Wendland C2.
template <int KER>
__device__ __forceinline__ float kw(float r, const CaseDev& c) {
  float q = r * c.inv_h;
  if (KER == 0) {
    float q1 = fmaxf(0.0f, 1.0f - q), q2 = fmaxf(0.0f, 2.0f - q), q3 = fmaxf(0.0f, 3.0f - q);
    float a = q3 * q3, b = q2 * q2, d = q1 * q1;
    return c.sigma * (a * a * q3 - 6.0f * (b * b * q2) + 15.0f * (d * d * q1));
  } else {
    float q1 = fmaxf(0.0f, 1.0f - 0.5f * q);
    float a = q1 * q1;
    return c.sigma * (a * a * (2.0f * q + 1.0f));
  }
}

template <int KER>
__device__ __forceinline__ float kdw(float r, const CaseDev& c) {
  float q = r * c.inv_h;
  if (KER == 0) {
    float q1 = fmaxf(0.0f, 1.0f - q), q2 = fmaxf(0.0f, 2.0f - q), q3 = fmaxf(0.0f, 3.0f - q);
    float a = q3 * q3, b = q2 * q2, d = q1 * q1;
    return c.dsigma * (a * a - 6.0f * (b * b) + 15.0f * (d * d));
  } else {
    float q1 = fmaxf(0.0f, 1.0f - 0.5f * q);
    return c.dsigma * (q * (q1 * q1 * q1));
  }
}

// Equations of state (eos.py:20-57).
__device__ __forceinline__ float eos_p(float rho, const CaseDev& c) {
  if (c.eos == SPH_EOS_TAIT) {
    float x = rho / c.rho_ref;
    if (c.gamma != 1.0f) x = powf(x, c.gamma);
    return c.p_ref * (x - 1.0f) + c.p_bg;
  }
  return c.rie_k * (rho - c.rho_ref) + c.p_bg;
}

__device__ __forceinline__ float eos_rho(float p, const CaseDev& c) {
  if (c.eos == SPH_EOS_TAIT) {
    float x = (p + c.p_ref - c.p_bg) / c.p_ref;
    if (c.gamma != 1.0f) x = powf(x, c.inv_gamma);
    return c.rho_ref * x;
  }
  return (p - c.p_bg) / c.rie_k + c.rho_ref;
}

// External acceleration g_ext_fn(r) of the case (cases/*.py).
template <int DIM>
__device__ __forceinline__ float3 g_ext(const CaseDev& c, const float4& r, const float* garr,
                                        int orig) {
  float3 g = make_float3(0.f, 0.f, 0.f);
  if (c.g_kind == SPH_GEXT_CONST) {
    g = make_float3(c.g[0], c.g[1], c.g[2]);
  } else if (c.g_kind == SPH_GEXT_BAND_X) {
    if (r.y < c.g_hi && r.y > c.g_lo) g.x = c.g[0];
  } else if (c.g_kind == SPH_GEXT_REVERSE_X) {
    g.x = r.y > c.g_hi ? -c.g[0] : c.g[0];
  } else if (c.g_kind == SPH_GEXT_ARRAY && garr) {
    g.x = garr[(size_t)orig * DIM + 0];
    g.y = garr[(size_t)orig * DIM + 1];
    if (DIM == 3) g.z = garr[(size_t)orig * DIM + 2];
  }
  return g;
}

// bc_fn on a velocity-like vector (u or v) of a particle with `tag`.
__device__ __forceinline__ float3 bc_vel(float3 u, int tag, const CaseDev& c) {
  if (c.bc_kind == SPH_BC_SOLID_ZERO || c.bc_kind == SPH_BC_SOLID_ZERO_P) {
    if (tag == SOLID_WALL) u = make_float3(0.f, 0.f, 0.f);
  } else if (c.bc_kind == SPH_BC_LID) {
    if (tag == SOLID_WALL) u = make_float3(0.f, 0.f, 0.f);
    if (tag == MOVING_WALL) u = make_float3(c.u_lid[0], c.u_lid[1], c.u_lid[2]);
  } else if (c.bc_kind == SPH_BC_HT) {
    if (tag == SOLID_WALL || tag == DIRICHLET_WALL) u = make_float3(0.f, 0.f, 0.f);
  }
  return u;
}
// bc_fn on an acceleration (dudt or dvdt).
__device__ __forceinline__ float3 bc_acc(float3 a, int tag, const CaseDev& c) {
  if (c.bc_kind == SPH_BC_SOLID_ZERO || c.bc_kind == SPH_BC_SOLID_ZERO_P) {
    if (tag == SOLID_WALL) a = make_float3(0.f, 0.f, 0.f);
  } else if (c.bc_kind == SPH_BC_LID) {
    if (tag == SOLID_WALL || tag == MOVING_WALL) a = make_float3(0.f, 0.f, 0.f);
  } else if (c.bc_kind == SPH_BC_HT) {
    if (tag == SOLID_WALL || tag == DIRICHLET_WALL) a = make_float3(0.f, 0.f, 0.f);
  }
  return a;
}
// bc_fn on the temperature and its rate (cases/ht.py:176-211), `x` the
// particle's (new) first coordinate.
__device__ __forceinline__ void bc_temp(float& T, float& dTdt, int tag, float x,
                                        const CaseDev& c) {
  if (c.bc_kind != SPH_BC_HT) return;
  if ((tag == FLUID && x < c.bc_x[0]) || tag == SOLID_WALL) {
    T = c.bc_T[0];
    dTdt = 0.f;
  } else if (tag == DIRICHLET_WALL) {
    T = c.bc_T[1];
    dTdt = 0.f;
  }
  if (tag == FLUID && x > c.bc_x[1]) dTdt = 0.f;
}
__device__ __forceinline__ float bc_p(float p, int tag, const CaseDev& c) {
  return (c.bc_kind == SPH_BC_SOLID_ZERO_P && tag == SOLID_WALL) ? 0.0f : p;
}

// Cell of a position: hash = sum(int32(r / cell_size) * mult)
// (jax_md/partition.py:367-368), axes with a single cell contribute 0.
template <int DIM>
__device__ __forceinline__ int cell_hash(const float4& r, const CaseDev& c, unsigned* status) {
  float rr[3] = {r.x, r.y, r.z};
  int h = 0;
  bool finite = true;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    finite &= isfinite(rr[d]);
    int ix = c.nc[d] > 1 ? __float2int_rz(__fdiv_rn(rr[d], c.cell_size[d])) : 0;
    h += ix * c.mult[d];
  }
  if (!finite) {
    atomicOr(status, SPH_ERR_NONFINITE);
    h = 0;
  } else if (h < 0 || h >= c.ncell) {
    atomicOr(status, SPH_WARN_BOX_EDGE);
    h = h < 0 ? 0 : c.ncell - 1;
  }
  return h;
}

// Visit the candidate senders of a receiver in cell `cell_local` at ri as
// ranges [j0, j1) of the cell-sorted order, f(j0, j1, s), where s (per axis
// -L, 0 or +L) is the periodic shift that maps the range's particles to their
// image next to the receiver. The walk covers rad[d] cells on each side of the
// receiver's cell along every axis (the whole axis where rad = 0): with
// c.rad, a superset of the reference's 3^d-cell candidates that are within
// the cutoff (jax_md/partition.py:832-856); with c.vrad, of those within the
// Verlet radius. Cells along x are contiguous in the sorted order, so each
// (y, z) row is one range, or two where it wraps.
// TRIM (fast cases): a row whose nearest point lies beyond sqrt(trim_r2) is
// skipped and the x extent of the others is cut to the sphere's chord; the
// bounds are lowered by trim_m, so no particle within that sphere is ever
// left out.
template <int DIM, bool TRIM, typename F>
__device__ __forceinline__ void walk_rows(const CaseDev& c, int cell_local, const float4& ri,
                                          const int* __restrict__ start, const int* rad,
                                          float trim_r2, F&& f) {
  const int nx = c.nc[0], ny = c.nc[1], nz = (DIM == 3) ? c.nc[2] : 1;
  const int cx = cell_local % nx;
  const int t = cell_local / nx;
  const int cy = t % ny;
  const int cz = (DIM == 3) ? t / ny : 0;
  const int* cs = start + c.cell_off;
  const int rx = rad[0], ry = rad[1];
  const int rz = (DIM == 3) ? rad[2] : 0;
  for (int dz = -rz; dz <= rz; ++dz) {
    int zz = cz + dz;
    float sz = 0.f;
    if (zz < 0) { zz += nz; sz = -c.box[2]; }
    else if (zz >= nz) { zz -= nz; sz = c.box[2]; }
    float gz2 = 0.f;
    if (TRIM && DIM == 3 && dz != 0) {
      const float g = (dz > 0 ? (float)(cz + dz) * c.cell_size[2] - ri.z
                              : ri.z - (float)(cz + dz + 1) * c.cell_size[2]) - c.trim_m;
      gz2 = g > 0.f ? g * g : 0.f;
    }
    for (int dy = -ry; dy <= ry; ++dy) {
      int yy = cy + dy;
      float sy = 0.f;
      if (yy < 0) { yy += ny; sy = -c.box[1]; }
      else if (yy >= ny) { yy -= ny; sy = c.box[1]; }
      const int row = (zz * ny + yy) * nx;
      // x cells [xa, xb] of this row, unwrapped
      int xa = cx - rx, xb = cx + rx;
      if (TRIM) {
        float g2 = gz2;
        if (dy != 0) {
          const float g = (dy > 0 ? (float)(cy + dy) * c.cell_size[1] - ri.y
                                  : ri.y - (float)(cy + dy + 1) * c.cell_size[1]) - c.trim_m;
          if (g > 0.f) g2 += g * g;
        }
        if (g2 >= trim_r2) continue;
        const float w = sqrtf(trim_r2 - g2) + c.trim_m;
        // the chord's cells, clamped in floating point first: a non-finite
        // position (NaN fails every test, +-inf saturates) keeps the
        // untrimmed row instead of converting an out-of-range bound
        const float lo = floorf((ri.x - w) * c.inv_cs[0]);
        const float hi = floorf((ri.x + w) * c.inv_cs[0]);
        const int ta = (int)fminf(fmaxf(lo, (float)xa), (float)xb);
        const int tb = (int)fminf(fmaxf(hi, (float)xa), (float)xb);
        xa = ta;
        xb = tb;
      }
      // up to two ranges (the second where the row wraps); the visitor is
      // instantiated once, inside the loop
      int a0, b0, a1 = row, b1 = row;
      float s1 = 0.f;
      if (rx == 0) {
        a0 = row; b0 = row + nx;
      } else if (xa < 0) {
        a0 = row; b0 = row + xb + 1; a1 = row + xa + nx; b1 = row + nx; s1 = -c.box[0];
      } else if (xb >= nx) {
        a0 = row + xa; b0 = row + nx; a1 = row; b1 = row + xb - nx + 1; s1 = c.box[0];
      } else {
        a0 = row + xa; b0 = row + xb + 1;
      }
#pragma unroll 1
      for (int r = 0; r < 2; ++r) {
        const int a = r ? a1 : a0, e = r ? b1 : b0;
        if (e > a) f(cs[a], cs[e], make_float3(r ? s1 : 0.f, sy, sz));
      }
    }
  }
}

// Occupancy of the reference's cell that contains fine cell `cell_local`:
// the sum over its sub[0] x sub[1] x sub[2] fine cells.
template <int DIM>
__device__ __forceinline__ int ref_cell_occupancy(const CaseDev& c, int cell_local,
                                                  const int* __restrict__ start) {
  const int* cs = start + c.cell_off;
  const int nx = c.nc[0], ny = c.nc[1];
  const int cx = cell_local % nx;
  const int t = cell_local / nx;
  const int cy = t % ny;
  const int cz = (DIM == 3) ? t / ny : 0;
  const int bx = cx - cx % c.sub[0], by = cy - cy % c.sub[1];
  const int sz = (DIM == 3) ? c.sub[2] : 1;
  const int bz = cz - cz % sz;
  int occ = 0;
  for (int oz = 0; oz < sz; ++oz)
    for (int oy = 0; oy < c.sub[1]; ++oy) {
      const int row = ((bz + oz) * ny + by + oy) * nx + bx;
      occ += cs[row + c.sub[0]] - cs[row];
    }
  return occ;
}

// int32(r / cs), the cell hash's index along an axis of cell size cs: r * inv_cs
// lies within 1.5 * 2^-23 (relative) of the correctly rounded quotient, so its
// floor is the hash's unless it lies that close to an integer; only then (and
// for negative or non-finite r) the division decides.
__device__ __forceinline__ int hash_index(float r, float cs, float inv_cs) {
  const float q = r * inv_cs;
  const float f = q - floorf(q);
  const float tol = fmaxf(q, 1.0f) * 4.8e-7f;
  if (q >= 0.f && f > tol && f < 1.0f - tol) return (int)q;
  return __float2int_rz(__fdiv_rn(r, cs));
}

// Index of the reference's cell of r within its case (the reference's hash,
// jax_md/partition.py:367-368): the binned cell coordinates divided by sub,
// clamped into the grid. Returns -1 for a non-finite position.
template <int DIM>
__device__ __forceinline__ int ref_cell_hash(const float4& r, const CaseDev& c) {
  const float rr[3] = {r.x, r.y, r.z};
  int h = 0, mult = 1;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    if (!isfinite(rr[d])) return -1;
    // sub is 1 or 2 (fine cells of half the reference's size): division by
    // it is a shift, and the fine index int32(r / cs) is hash_index's
    const int sh = c.sub[d] - 1;
    const int n = c.nc[d] >> sh;
    int ix = c.nc[d] > 1 ? hash_index(rr[d], c.cell_size[d], c.inv_cs[d]) >> sh : 0;
    ix = ix < 0 ? 0 : (ix >= n ? n - 1 : ix);
    h += ix * mult;
    mult *= n;
  }
  return h;
}

// Whether sender b lies in one of the 3^d reference cells around receiver
// a's (per axis the same cell or a neighbour, periodically): the reference
// tests only those senders (jax_md/partition.py:832-856). Fast cases walk
// finer cells a little beyond them, so a pair at the cutoff distance whose
// reference cells are two apart -- possible where the reference's cell is the
// cutoff to within rounding -- must not become an edge. Pairs clearly inside
// the cutoff are always adjacent (the band's margin exceeds the hash's
// rounding), so only the band's candidates take this test.
//
template <int DIM>
__device__ __forceinline__ bool ref_adjacent(const float4& a, const float4& b, const CaseDev& c) {
  const float pa[3] = {a.x, a.y, a.z}, pb[3] = {b.x, b.y, b.z};
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const int sh = c.sub[d] - 1;  // sub is 1 or 2
    const int n = c.nc[d] >> sh;
    if (n < 3) continue;
    int ia = hash_index(pa[d], c.cell_size[d], c.inv_cs[d]) >> sh;
    int ib = hash_index(pb[d], c.cell_size[d], c.inv_cs[d]) >> sh;
    ia = ia < 0 ? 0 : (ia >= n ? n - 1 : ia);
    ib = ib < 0 ? 0 : (ib >= n ? n - 1 : ib);
    const int k = ia > ib ? ia - ib : ib - ia;
    if (k > 1 && k < n - 1) return false;
  }
  return true;
}

// The reference metric, out of line: only candidates in the narrow band
// around the cutoff (or every candidate of a case without the fast test)
// reach it, so the hot loop stays small.
//
// The band's pairs are at the cutoff, i.e. at most about one reference cell
// apart: an axis along which the displacement d is clearly shorter than the
// reference cell (by more than the hash's rounding, 4 n + 8 ulp of the cell
// index for n cells) cannot separate them by two cells, and only the other
// axes need the cell indices.
template <int DIM>
__device__ __forceinline__ bool ref_adjacent_d(const float4& a, const float4& b, const float3& d,
                                               const CaseDev& c) {
  const float pa[3] = {a.x, a.y, a.z}, pb[3] = {b.x, b.y, b.z}, pd[3] = {d.x, d.y, d.z};
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    const int sh = c.sub[k] - 1;  // sub is 1 or 2
    const int n = c.nc[k] >> sh;
    if (n < 3) continue;
    const float cref = c.cell_size[k] * (float)c.sub[k];
    if (fabsf(pd[k]) < cref * (1.0f - (float)(4 * n + 8) * 1.2e-7f)) continue;
    int ia = hash_index(pa[k], c.cell_size[k], c.inv_cs[k]) >> sh;
    int ib = hash_index(pb[k], c.cell_size[k], c.inv_cs[k]) >> sh;
    ia = ia < 0 ? 0 : (ia >= n ? n - 1 : ia);
    ib = ib < 0 ? 0 : (ib >= n ? n - 1 : ib);
    const int s = ia > ib ? ia - ib : ib - ia;
    if (s > 1 && s < n - 1) return false;
  }
  return true;
}

template <int DIM>
__device__ __noinline__ bool exact_edge(float4 ri, float4 rj, const CaseDev* c) {
  const float3 d = pdisp3<DIM>(rj, ri, *c);
  if (!(sqd<DIM>(d) < c->cutoff_sq)) return false;
  return !c->fast || ref_adjacent_d<DIM>(ri, rj, d, *c);
}

// Membership as the list's backend defines it, for the emitted edge lists and
// their counts: the matscipy backend's float64 rule or the reference metric.
// The passes' per-step sums keep the float32 test (exact_edge): the two rules
// differ only for a pair at the cutoff distance, where W and W' vanish, so no
// sum changes. (A float64 branch inside exact_edge makes every caller of it
// save more registers: the hot loops would spill.)
template <int DIM>
__device__ __noinline__ bool list_edge(float4 ri, float4 rj, const CaseDev* c) {
  if (c->f64_metric) return is_edge_f64<DIM>(ri, rj, *c);
  return is_edge<DIM>(ri, rj, *c) && (!c->fast || ref_adjacent<DIM>(ri, rj, *c));
}

// Minimum-image r_i - r_j of a pair already known to be an edge.
template <int DIM>
__device__ __forceinline__ void pair_dr(const float4& ri, const float4& rj, const CaseDev& c,
                                        float3& dr, float& d2) {
  if (c.fast) {
    dr.x = ri.x - rj.x;
    dr.y = ri.y - rj.y;
    dr.z = (DIM == 3) ? ri.z - rj.z : 0.f;
    dr.x = fmaf(-c.box[0], rintf(dr.x * c.inv_box[0]), dr.x);
    dr.y = fmaf(-c.box[1], rintf(dr.y * c.inv_box[1]), dr.y);
    if (DIM == 3) dr.z = fmaf(-c.box[2], rintf(dr.z * c.inv_box[2]), dr.z);
    d2 = dr.x * dr.x + dr.y * dr.y + dr.z * dr.z;
  } else {
    dr = pdisp3<DIM>(ri, rj, c);
    d2 = sqd<DIM>(dr);
  }
}

// Membership of edge (receiver ri, sender rj) for a candidate whose periodic
// image is not known from a walk (Verlet list, walk of a past binning): the
// minimum-image squared distance against the band [lo, hi), the reference
// metric inside it. That distance differs from the reference metric by no
// more than the shifted one does, so the band of the fast test holds. A case
// without the fast test takes the reference metric for every candidate.
template <int DIM>
__device__ __forceinline__ bool edge_mi(const float4& ri, const float4& rj, float lo, float hi,
                                        const CaseDev& c, const CaseDev* cp) {
  if (!c.fast) return exact_edge<DIM>(ri, rj, cp);
  float3 dr;
  float d2;
  pair_dr<DIM>(ri, rj, c, dr, d2);
  bool in = d2 < lo;
  if (!in && d2 < hi) in = exact_edge<DIM>(ri, rj, cp);
  return in;
}

// edge_mi that also returns the squared distance pair_dr gives the pair.
template <int DIM>
__device__ __forceinline__ bool edge_mi_d2(const float4& ri, const float4& rj, float lo,
                                           float hi, const CaseDev& c, const CaseDev* cp,
                                           float& d2) {
  float3 dr;
  pair_dr<DIM>(ri, rj, c, dr, d2);
  if (!c.fast) return exact_edge<DIM>(ri, rj, cp);
  bool in = d2 < lo;
  if (!in && d2 < hi) in = exact_edge<DIM>(ri, rj, cp);
  return in;
}

// Compensated accumulation (Kahan) selected at compile time.
template <bool KAHAN>
struct Acc {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    if (KAHAN) {
      float y = x - c;
      float t = s + y;
      c = (t - s) - y;
      s = t;
    } else {
      s += x;
    }
  }
};

// ------------------------------------------------------------------ wall normals
// A static, 5x finer layer of points along the walls (utils.py:197-275): each
// step the wall particles' normals point to their nearest layer point.
// Points are binned in a grid of at least the search radius (cs >= cutoff).
struct WallLayer {
  const float4* pts;  // (x, y, z, layer index as int bits), sorted by cell
  const int* start;   // [ncell + 1] cell offsets into pts
  int n;              // layer points (0: no recomputation)
  int nc[3];
  float cs[3];
  float off[3];       // wall particles are searched at r - off
  float cut2;         // squared search radius
};

// The displacement from wall particle position `r` to its nearest layer
// point within the search radius, normalised: nw = dr / (|dr| + eps); zero
// when none is within it (compute_nws_jax_wrapper, utils.py:239-270). The
// reference's candidates are the layer points of a dense neighbour list with
// index > 0 only (it compares the list index with the number of walls
// strictly), so layer point 0 never counts; among equally near points the
// one with the lowest index wins.
template <int DIM>
__device__ __forceinline__ float4 wall_normal(const float4& r, const WallLayer& w,
                                              const CaseDev& c) {
  const float4 p = make_float4(__fsub_rn(r.x, w.off[0]), __fsub_rn(r.y, w.off[1]),
                               DIM == 3 ? __fsub_rn(r.z, w.off[2]) : 0.f, 0.f);
  int cell[3] = {0, 0, 0};
  const float pc[3] = {p.x, p.y, p.z};
  for (int d = 0; d < DIM; ++d) {
    float x = pc[d] - c.box[d] * floorf(pc[d] / c.box[d]);  // wrap for binning only
    int k = (int)(x / w.cs[d]);
    cell[d] = k < 0 ? 0 : (k >= w.nc[d] ? w.nc[d] - 1 : k);
  }
  float best = INFINITY;
  int best_idx = INT_MAX;
  float3 bdr = make_float3(0.f, 0.f, 0.f);
  const int span[3] = {w.nc[0] < 3 ? w.nc[0] : 3, w.nc[1] < 3 ? w.nc[1] : 3,
                       DIM == 3 ? (w.nc[2] < 3 ? w.nc[2] : 3) : 1};
  for (int a = 0; a < span[0]; ++a)
    for (int b = 0; b < span[1]; ++b)
      for (int e = 0; e < span[2]; ++e) {
        const int ox = w.nc[0] < 3 ? a : cell[0] + a - 1;
        const int oy = w.nc[1] < 3 ? b : cell[1] + b - 1;
        const int oz = DIM == 3 ? (w.nc[2] < 3 ? e : cell[2] + e - 1) : 0;
        const int cx = (ox + w.nc[0]) % w.nc[0], cy = (oy + w.nc[1]) % w.nc[1];
        const int cz = DIM == 3 ? (oz + w.nc[2]) % w.nc[2] : 0;
        const int q = cx + w.nc[0] * (cy + w.nc[1] * cz);
        for (int t = w.start[q]; t < w.start[q + 1]; ++t) {
          const float4 l = w.pts[t];
          const int li = __float_as_int(l.w);
          if (li == 0) continue;
          if (!(sqd<DIM>(pdisp3<DIM>(p, l, c)) < w.cut2)) continue;
          const float3 dr = pdisp3<DIM>(l, p, c);
          const float dist = sqrtf(sqd<DIM>(dr));
          if (dist < best || (dist == best && li < best_idx)) {
            best = dist;
            best_idx = li;
            bdr = dr;
          }
        }
      }
  if (best_idx == INT_MAX) return make_float4(0.f, 0.f, 0.f, 0.f);
  const float den = best + kEps;
  return make_float4(bdr.x / den, bdr.y / den, bdr.z / den, 0.f);
}

// ------------------------------------------------------------------ launchers
struct Workspace;  // defined in sph_capi.cu

struct LaunchCtx {
  cudaStream_t stream;
  int dim, kernel, solver;
  int rho_evol, bc_trick, free_slip, mask_self, kahan;
  int rho_renorm;         // renormalise the evolved density
  int heat;               // heat conduction
  WallLayer layer;        // wall normals recomputed in the kick (layer.n > 0)
  long long N;
  int n_cases;
  const CaseDev* cases;   // device
  unsigned* status;       // device
  int* nbr;               // per-step neighbour list [kmax][N]
  int* nbr_cnt;           // neighbours per particle (self excluded)
  int kmax;
  int* vl;                // Verlet candidates [kv][N], ascending original index
  int* vcnt;              // candidates per particle (may exceed kv)
  int kv;
  float4* rref;           // positions at the last rebuild
  int* cref_count;        // per-step occupancy of the reference's cells
  unsigned* vflag;        // a rebuild is due
  int canonical;          // candidate lists in ascending original index
  int* inv;               // sorted position of every original index (last binning)
  float4* R4e;            // evolved density before renormalisation (rho_renorm)
  float4* dscr;           // delta-SPH density scratch: 5 planes of N float4
  int block;              // threads per block of the forward passes (<= 256)
  int lean;               // lean passes (sph_lean.cu): 0 no, 1 16-bit lists, 2 32-bit
  int force_variant;      // SPH_FORCE_*: how the lean force pass reads its senders
  CaseDev c1;             // the single case (the lean passes take it by value)
  int* launches;          // optional host counter of kernel launches
  cudaEvent_t* ev;        // optional phase events: bin start, bin end, density end,
                          // wall end, force end
};

inline void count_launch(const LaunchCtx& L, int k = 1) {
  if (L.launches) *L.launches += k;
}
inline void mark(const LaunchCtx& L, int i) {
  if (L.ev) cudaEventRecord(L.ev[i], L.stream);
}

// sph_sort.cu
// Load a state given in original order (into a binning's sorted slots with
// `inv`, raising `changed` when a position differs from the one there).
void launch_pack(const LaunchCtx& L, const SphStateView& s, Buffers out,
                 const long long* case_off_dev, const int* inv = nullptr,
                 unsigned* changed = nullptr);
// Write the state back in original order; with `inv` (the binning's inverse
// permutation) by original index, gathering from the sorted buffers and
// writing coalesced.
void launch_unpack(const LaunchCtx& L, Buffers in, const float4* R4, SphStateView& s,
                   bool from_forward, bool apply_bc, const float* ref = nullptr,
                   float thr_sq = 0.f, const int* inv = nullptr);
// `copy_src`: the resident set, copied into `in` by the hashing kernel first
// (a rebuild's scratch copy).
void launch_bin(const LaunchCtx& L, Buffers in, Buffers out, const float4* R4, int* cellid,
                int* count, int* start, int* keyc, int* keys, int* tsrc, int* tkey, int* tcell,
                int* scan_tmp, long long total_cells, bool drift, bool from_forward,
                bool apply_bc, float4* rref, const Buffers* copy_src = nullptr);
// In-place kick-drift of a step on the resident buffers, with the per-step
// reference-cell occupancy test and the rebuild test.
void launch_kick(const LaunchCtx& L, Buffers b, const float4* R4, long long ref_cells,
                 bool from_forward, bool apply_bc);
int launch_scan(cudaStream_t st, const int* in, int* out, long long n, int* tmp);
// Exclusive scan of n ints into 64-bit offsets (tmp: scan_tmp_ints(n) ints,
// 8-byte aligned).
int launch_scan64(cudaStream_t st, const int* in, long long* out, long long n, int* tmp);
void launch_edges(const LaunchCtx& L, Buffers b, const int* cellid, const int* start,
                  int* rowcnt, long long* rowoff, int* scan_tmp, int32_t* idx, long long capacity,
                  long long* count_dev);
void launch_row_counts(const LaunchCtx& L, Buffers b, const int* cellid, const int* start,
                       int* rowcnt);
// Per case: largest reference-cell occupancy and edge count of the binning.
void launch_alloc_stats(const LaunchCtx& L, Buffers b, const int* cellid, const int* start,
                        const int* rowcnt, int* case_max, unsigned long long* case_edges);
void launch_diagnostics(const LaunchCtx& L, Buffers b, const float4* R4, bool from_forward,
                        bool apply_bc, double* out);
// Per original index, the last forward pass's neighbour count (self pair
// included unless masked; padding 0).
void launch_neighbour_counts(const LaunchCtx& L, Buffers b, int32_t* counts);
// Flag bit on a step-list count: the receiver's senders did not fit the
// list's format (the lean passes); the count itself is below it.
constexpr int kCountFlag = 1 << 30;

// sph_forward.cu
// Verlet candidate lists of the current binning.
void launch_verlet(const LaunchCtx& L, Buffers b, const int* cellid, const int* start);
// One-time kernel attributes (shared-memory opt-in); returns a CUDA error.
cudaError_t prepare_kernels(int kv);
// phases: 1 the density passes and the wall BC, 2 the force pass, 3 both.
void launch_forward(const LaunchCtx& L, Buffers b, const float4* R4, float4* R4w, float4* UT4,
                    const int* cellid, const int* start, unsigned long long* edgecnt,
                    const float* g_arr, bool apply_bc, bool has_walls, int phases = 3);

// sph_lean.cu: the lean candidate build and passes (one periodic case with
// the fast test, standard SPH, density summation, no wall BC, no heat, cell
// order). Their lists live in the buffers of the 32-bit lists. lean_config:
// 0 not served, 1 served with 16-bit list offsets, 2 with 32-bit indices.
int lean_config(const SphConfig& cfg, int n_cases, const CaseDev& c0);
void launch_verlet_lean(const LaunchCtx& L, Buffers b, const int* cellid, const int* start);
void launch_forward_lean(const LaunchCtx& L, Buffers b, float4* R4, const int* cellid,
                         const int* start, unsigned long long* edgecnt, const float* g_arr,
                         bool apply_bc, int phases);

// sph_delta.cu (after the density pass has written the step's neighbour list)
// delta-SPH density evolution into Rout (rho, p, drho/dt, eta).
void launch_delta_density(const LaunchCtx& L, Buffers b, float4* Rout, const int* cellid,
                          const int* start, int sph_gwbc);
// Density renormalisation of the evolved densities in Rin into Rout.
void launch_renorm(const LaunchCtx& L, Buffers b, const float4* Rin, float4* Rout,
                   const int* cellid, const int* start, int sph_gwbc);

size_t scan_tmp_ints(long long n);

// sph_adjoint.cu: the recorded forward data of one step and the reverse's
// per-step scratch (sorted order of that step).
struct AdjTape {
  const int* orig;
  const float4 *P4, *U4, *V4, *R4;
  const int* meta;
  const int *nbr, *cnt;
};
struct AdjScratch {
  float4 *F1, *F2, *F3, *WB, *WU, *WV, *GU, *GV;
};
// Copy the step just taken into a tape slot (one kernel).
void launch_tape_record(const LaunchCtx& L, Buffers b, const float4* R4, int* t_orig,
                        float4* t_P4, float4* t_U4, float4* t_V4, float4* t_R4, int* t_meta,
                        int* t_nbr, int* t_cnt);
// Reverse of one recorded step: lr, lu in place, la/lb (adjoints of the
// step's dudt/dvdt outputs) to la_out/lb_out (those of its inputs). `walls`:
// the generalized wall BC ran in the step.
void launch_adjoint(const LaunchCtx& L, const AdjTape& t, const AdjScratch& s, const float* la,
                    const float* lb, float* la_out, float* lb_out, float* lr, float* lu,
                    int walls);

// sph_capi.cu: per-case device constants from the ABI parameters; returns
// non-zero and sets `err` on invalid input.
int make_case(const SphConfig& cfg, const SphCase& in, long long p_off, long long cell_off,
              CaseDev& c, std::string& err, bool fine_cells = true);
// sph_capi.cu: the message sph_last_error returns on this host thread.
void set_last_error(const std::string& msg);
// sph_capi.cu: called from the catch clause of an entry point; records the
// in-flight C++ exception as the last error and returns SPH_ERR_HOST, so no
// exception crosses the C ABI.
int host_error() noexcept;

}  // namespace sph
