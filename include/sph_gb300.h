/*
 * sph_gb300.h -- C ABI of the GB300 (sm_103a) jax-sph hot path.
 *
 * One handle owns the device workspace for a set of independent SPH cases
 * ("instances", one for the plain path, many for the batched form) that share
 * one dimension, kernel, solver and boundary-treatment configuration. All
 * particle data crossing this ABI lives in device memory owned by the caller,
 * laid out exactly like the reference's state dict (one row per particle,
 * row-major (N, dim) float32 for vectors). The library never frees caller
 * memory; only sph_create allocates.
 *
 * Every entry point returns an int status: 0 on success, otherwise a
 * combination of the SPH_ERR_* bits below. Data-dependent conditions found on
 * the device (the reference's PartitionErrorCode bits, non-finite values) are
 * accumulated in a device status word and read with sph_read_status, the way
 * the reference polls NeighborList.error (jax_md/partition.py:453-499,
 * jax_sph/simulate.py:120-128). No exception crosses the ABI. Calls are
 * stream-ordered on the stream passed as `stream` (a cudaStream_t, 0 = legacy
 * default stream). A handle is thread-compatible: one host thread at a time.
 *
 * Reference interfaces replaced (paths within tumaer/jax-sph):
 *   partition.neighbor_list(...).allocate / .update  jax_sph/partition.py:492-571,
 *       jax_sph/jax_md/partition.py:723-1026        -> sph_nl_allocate, sph_nl_update,
 *                                                       sph_nl_edges
 *   WCSPH(...).forward_wrapper()(state, neighbors)   jax_sph/solver.py:613-951
 *                                                    -> sph_forward
 *   si_euler(...)(dt, state, neighbors)              jax_sph/integrator.py:8-58
 *                                                    -> sph_step
 */
#ifndef SPH_GB300_H
#define SPH_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_ABI_VERSION 7

/* Reference PartitionErrorCode bits (jax_sph/jax_md/partition.py:453-457). */
#define SPH_NEIGHBOR_LIST_OVERFLOW 0x1u
#define SPH_CELL_LIST_OVERFLOW 0x2u
#define SPH_CELL_SIZE_TOO_SMALL 0x4u
#define SPH_MALFORMED_BOX 0x8u
/* Library bits. */
#define SPH_ERR_INVALID_ARG 0x100u
#define SPH_ERR_CUDA 0x200u
#define SPH_ERR_TIMEOUT 0x400u
#define SPH_ERR_NONFINITE 0x800u
/* A position hashed outside the cell grid (exactly on the upper box face);
 * it is clamped into the last cell. */
#define SPH_WARN_BOX_EDGE 0x1000u
/* sph_advance: a particle moved beyond the neighbour list's threshold. */
#define SPH_INFO_MOVED 0x2000u
/* A host-side failure inside the library (host memory exhausted or another
 * C++ exception), returned instead of letting it cross the ABI. */
#define SPH_ERR_HOST 0x4000u

enum { SPH_KERNEL_QSK = 0, SPH_KERNEL_WC2K = 1 };   /* jax_sph/kernel.py:51-103 */
/* jax_sph/solver.py:676-694; DELTA: the standard SPH acceleration plus the
 * delta-SPH diffusive term (solver.py:259-313), with summation density or the
 * delta-SPH density evolution (solver.py:33-105) */
enum { SPH_SOLVER_SPH = 0, SPH_SOLVER_RIE = 1, SPH_SOLVER_DELTA = 2 };
enum { SPH_EOS_TAIT = 0, SPH_EOS_RIEMANN = 1 };     /* jax_sph/eos.py:20-57 */

/* External acceleration g_ext_fn(r) of the cases on the path. */
enum {
  SPH_GEXT_ZERO = 0,   /* TGV, LDC (cases/tgv.py:53, cases/ldc.py:124) */
  SPH_GEXT_CONST = 1,  /* g everywhere (DB: (0,-g), cases/db.py:123-126) */
  SPH_GEXT_BAND_X = 2, /* g.x where band_lo < y < band_hi (PF, cases/pf.py:122-131) */
  SPH_GEXT_ARRAY = 3,  /* per-particle array from SphStateView.g_ext */
  SPH_GEXT_REVERSE_X = 4 /* g.x where y <= band_hi, -g.x above it (RPF, cases/rpf.py:58-63) */
};

/* Boundary condition bc_fn(state) applied after the forward pass by a step. */
enum {
  SPH_BC_NONE = 0,          /* TGV (cases/tgv.py:56-57) */
  SPH_BC_SOLID_ZERO = 1,    /* u,v,dudt,dvdt = 0 on SOLID_WALL (PF, cases/pf.py:133-146) */
  SPH_BC_SOLID_ZERO_P = 2,  /* as above and p = 0 (DB, cases/db.py:128-142) */
  SPH_BC_LID = 3,           /* SOLID_WALL at rest, MOVING_WALL at u_lid (LDC, cases/ldc.py:127-144) */
  SPH_BC_HT = 4             /* heat transfer over a plate (cases/ht.py:176-211): SOLID_WALL and
                               DIRICHLET_WALL at rest; T = bc_T[0] (dTdt = 0) on SOLID_WALL and
                               on fluid with x < bc_x[0], T = bc_T[1] on DIRICHLET_WALL,
                               dTdt = 0 on fluid with x > bc_x[1] */
};

/* Configuration shared by every case of a handle. */
typedef struct SphConfig {
  int32_t dim;            /* 2 or 3 */
  int32_t kernel;         /* SPH_KERNEL_* */
  int32_t solver;         /* SPH_SOLVER_* */
  int32_t is_rho_evol;    /* density evolution instead of summation */
  int32_t is_bc_trick;    /* generalized wall boundary condition */
  int32_t is_free_slip;
  int32_t mask_self;      /* exclude self pairs from the neighbour list */
  int32_t kahan;          /* compensated (Kahan) pair sums */
  int32_t fp64_positions; /* integrate positions in float64 (long rollouts); the
                             passes read them rounded to float32 */
  double capacity_multiplier; /* neighbour/cell capacity factor (reference 1.25) */
  double verlet_skin;     /* candidate-list skin as a fraction of the cutoff, in
                             [0, 0.5]; 0 rebuilds the candidates every step. The
                             neighbour set of every step is the reference's either
                             way (each candidate takes the exact membership test) */
  int32_t canonical_order; /* sum pairs in ascending original index: results then
                              do not depend on the skin, the batching or when the
                              candidates were rebuilt (slower rebuilds and gathers);
                              0 sums in cell order, deterministic for a given run */
  int32_t is_rho_renorm;  /* density renormalisation after density evolution
                             (rho_renorm_fn, solver.py:167-173, :755-793) */
  int32_t is_heat_conduction; /* temperature equation (solver.py:591-610, :832-850) and
                                 the wall temperature BC (:518-526, :556-565) */
  int32_t nl_backend;     /* SPH_NL_JAXMD: the reference metric in float32 (jax_md);
                             SPH_NL_MATSCIPY: float64 minimum-image distance < cutoff
                             (partition.py:356-482, matscipy.neighbours) */
} SphConfig;

/* Neighbour-list backends. Particles tagged SPH_TAG_PAD (-1, Tag.PAD_VALUE,
 * utils.py:25) pad a state to a fixed size: they are in no neighbour list
 * with either backend, and are kicked like any particle. */
enum { SPH_NL_JAXMD = 0, SPH_NL_MATSCIPY = 1 };
#define SPH_TAG_PAD (-1)

/* Per-case parameters (all in the reference's units). */
typedef struct SphCase {
  int64_t n;              /* particles of this case (cases are concatenated) */
  double box[3];          /* periodic box side lengths (cast to float32 like the reference) */
  double r_cutoff;        /* neighbour cutoff = kernel cutoff (3h QSK, 2h WC2K) */
  double dx;              /* lattice spacing (artificial-viscosity h_ab) */
  double h;               /* smoothing length */
  double dt;              /* si_euler time step (advance(dt, ...)) */
  double dt_solver;       /* WCSPH(dt=...) used by density evolution (solver.py:29, :790) */
  double tvf;             /* transport-velocity factor of si_euler */
  double c_ref;
  int32_t eos;            /* SPH_EOS_* */
  int32_t g_kind;         /* SPH_GEXT_* */
  int32_t bc_kind;        /* SPH_BC_* */
  int32_t pad0;
  double p_ref, rho_ref, p_bg, gamma, u_ref;
  double eta_limiter;     /* Riemann dissipation limiter, -1 = off */
  double artificial_alpha;
  double g[3];            /* SPH_GEXT_CONST / BAND_X magnitude vector */
  double g_band_lo, g_band_hi;
  double u_lid[3];
  double diff_alpha;      /* delta-SPH acceleration diffusion (DELTA solver) */
  double diff_delta;      /* delta-SPH density diffusion (DELTA, density evolution) */
  double bc_T[2];         /* SPH_BC_HT: reference and hot-wall temperature */
  double bc_x[2];         /* SPH_BC_HT: inflow below x = bc_x[0], outflow above bc_x[1] */
} SphCase;

/* Caller-owned device arrays in the reference state-dict layout
 * (jax_sph/case_setup.py:164-181). Vectors are (n, dim) row-major float32.
 * nw is needed only for the Riemann solver with the wall BC or free slip;
 * g_ext only with SPH_GEXT_ARRAY. Unused pointers may be NULL. */
typedef struct SphStateView {
  int64_t n;
  float* r;
  const int32_t* tag;
  float* u;
  float* v;
  float* dudt;
  float* dvdt;
  float* drhodt;
  float* rho;
  float* p;
  const float* mass;
  const float* eta;
  float* nw;              /* wall normals (n, dim); written by sph_advance and
                             sph_get_state when given (recomputed with a wall layer) */
  const float* g_ext;
  float* T;               /* temperature, its rate, conductivity, heat capacity (n,): */
  float* dTdt;            /*   required with is_heat_conduction, else ignored */
  const float* kappa;
  const float* Cp;
} SphStateView;

/* Capacities of the reference's two-phase neighbour list
 * (NeighborList.cell_list_capacity / max_occupancy). */
typedef struct SphNLCapacity {
  int64_t cell_capacity;  /* int(max cell occupancy * multiplier) */
  int64_t max_occupancy;  /* edge capacity: int(edge count * multiplier) */
  int64_t occupancy;      /* edges found at allocation */
  int64_t max_cell_occupancy;
} SphNLCapacity;

typedef struct SphHandle SphHandle;

/* Library ABI version (SPH_ABI_VERSION). */
int sph_abi_version(void);
/* Message of the last failing call on this host thread ("" if none). */
const char* sph_last_error(void);

/* Create a handle for `n_cases` cases sharing `cfg`. Allocates all device
 * workspace (the only allocating call). Replaces the host-side construction
 * done by neighbor_list(...) and WCSPH(...) (jax_sph/partition.py:492-571,
 * jax_sph/solver.py:616-700). */
int sph_create(const SphConfig* cfg, const SphCase* cases, int32_t n_cases,
               SphHandle** out);
int sph_destroy(SphHandle* h);
/* Replace the per-case physics parameters (dt, EOS, forcing, ...) of a
 * handle. The particle counts, boxes and cutoffs must stay unchanged
 * (they fix the workspace). */
int sph_update_cases(SphHandle* h, const SphCase* cases, int32_t n_cases);

/* Copy a state (original particle order) into the handle. */
int sph_set_state(SphHandle* h, const SphStateView* state, void* stream);
/* Write the handle's current state back in the original particle order. */
int sph_get_state(SphHandle* h, SphStateView* state, void* stream);

/* Neighbour list allocate (host-synchronous, like the reference's
 * non-jittable allocate, jax_md/partition.py:911-1001): bins the current
 * positions, measures the capacities and stores them in the handle. */
int sph_nl_allocate(SphHandle* h, int64_t extra_capacity, SphNLCapacity* cap_out,
                    void* stream);
/* Set capacities explicitly (a NeighborList carried over from elsewhere). */
int sph_nl_set_capacity(SphHandle* h, const SphNLCapacity* cap);
/* Neighbour list update with fixed capacities (jax_md/partition.py:1003-1026):
 * re-bins the current positions; sets SPH_CELL_LIST_OVERFLOW /
 * SPH_NEIGHBOR_LIST_OVERFLOW in the status word when a capacity is exceeded. */
int sph_nl_update(SphHandle* h, void* stream);
/* Emit the sparse edge list of the last binning into idx[2][capacity]
 * (row 0 = receiver/neighbour, row 1 = sender/particle, padding = n), sender
 * ascending, receivers ascending per sender. *count_dev (device int64)
 * receives the number of real edges; edges beyond `capacity` are dropped and
 * flag SPH_NEIGHBOR_LIST_OVERFLOW (jax_md/partition.py:885-909, :956-976). */
int sph_nl_edges(SphHandle* h, int32_t* idx, int64_t capacity, int64_t* count_dev,
                 void* stream);

/* WCSPH forward pass on the current state with the current binning
 * (jax_sph/solver.py:705-949): density, EOS, wall BC, forces, transport
 * velocity, artificial viscosity. No bc_fn is applied. */
int sph_forward(SphHandle* h, void* stream);
/* `nsteps` si_euler steps (jax_sph/integrator.py:22-56): kick, drift, neighbour
 * update (rebuilt every step), forward, bc_fn. Replays a CUDA graph. */
int sph_step(SphHandle* h, int32_t nsteps, void* stream);

/* One drop-in si_euler advance on caller buffers, the way the reference's
 * jitted advance(dt, state, neighbors) runs (jax_sph/integrator.py:22-56,
 * jax_sph/simulate.py:115-123): load `in`, kick, drift, neighbour update,
 * forward pass, bc_fn, and write the new state to `out` (which may alias
 * `in`). Arrays may be device memory or pinned host memory (read over the
 * host link by the load kernel, results copied back by DMA through device
 * staging the handle allocates on the first such call); pageable host
 * memory is rejected. `in->v` and, outside Riemann density evolution,
 * `in->p` are required but not read (the kick recomputes v); with a
 * summation `out->drhodt` may be NULL (the input's drho/dt is unchanged).
 * Then the status word is copied to `status_dev` (a device or pinned host
 * uint32) and cleared; it carries SPH_INFO_MOVED when some new position lies
 * farther than sqrt(threshold_sq) from `ref_r` (the list's reference
 * positions, (n, dim) float32; NULL skips the test) under the periodic
 * metric -- the reference's test for rebuilding the list
 * (jax_md/partition.py:1010-1018). With device arrays only, everything is
 * stream-ordered and the call does not wait; when a result or the status
 * word is in host memory, the call returns once it is there. */
int sph_advance(SphHandle* h, const SphStateView* in, SphStateView* out, const float* ref_r,
                float threshold_sq, uint32_t* status_dev, void* stream);

/* Moving walls (the integrator's nw_fn, jax_sph/integrator.py:33-34;
 * compute_nws_jax_wrapper, jax_sph/utils.py:197-275): from now on every step
 * sets, after the drift, the normal of each wall particle to the normalised
 * displacement from r - offset to its nearest point of `layer` (host (m, dim)
 * float32, the walls discretised 5x finer, in the same frame) within `cutoff`
 * (zero if none; layer point 0 is never a candidate, as in the reference;
 * ties go to the lowest index), and fluid normals to zero. m = 0 switches it
 * off. Single-case handles of a solver that keeps normals (Riemann or free
 * slip). Synchronous (host-side binning and upload). */
int sph_set_wall_layer(SphHandle* h, const float* layer, int64_t m, const double* offset,
                       double cutoff);

/* Threads per block of the density, wall and force passes (a multiple of 32
 * in [32, 256]; default 256). A tuning knob: results do not depend on it. */
int sph_set_block_size(SphHandle* h, int32_t threads);
/* How the force pass of the lean passes (sph_list_format 1 or 2) reads its
 * senders: SPH_FORCE_GATHER (default) gathers each sender's records from
 * global memory; SPH_FORCE_STAGED stages a block's senders in shared memory
 * one plane of cells at a time. Same pairs in the same order with the same
 * arithmetic: results do not depend on it. The generic passes ignore it. A
 * tuning knob: no reference interface corresponds to it. */
enum { SPH_FORCE_GATHER = 0, SPH_FORCE_STAGED = 1 };
int sph_set_force_variant(SphHandle* h, int32_t variant);
/* Kernel launches issued by one si_euler step of this handle (without a
 * candidate-list rebuild). */
int sph_step_launch_count(SphHandle* h, int32_t* count);
/* Which passes and list format serve this handle's steps: 0 the generic
 * passes (32-bit sender indices), 1 the lean passes with 16-bit offset
 * lists, 2 the lean passes with 32-bit index lists (the lean passes serve one
 * periodic case with standard SPH, density summation and no wall BC). A
 * diagnostic: no reference interface corresponds to it. */
int sph_list_format(SphHandle* h, int32_t* format);
/* Candidate-list rebuilds run so far by this handle's steps and the kernel
 * launches one rebuild adds to a step. Synchronizes `stream`. */
int sph_rebuild_stats(SphHandle* h, int64_t* rebuilds, int32_t* kernels_per_rebuild,
                      void* stream);
/* Run `nsteps` steps eagerly, timing their phases with CUDA events on
 * `stream` (where the kernels run): ms[0] kick-drift plus the candidate-list
 * rebuilds that fell in the steps, ms[1] density pass, ms[2] wall pass,
 * ms[3] force pass, ms[4] the kick-drift alone, ms[5] the rebuilds alone (the
 * sort and the candidate lists), each averaged per step; ms holds 6 floats.
 * Host-synchronous (the host reads the rebuild decision of each step); the
 * steps advance the state like sph_step. */
int sph_profile_step(SphHandle* h, int32_t nsteps, float* ms, void* stream);

/* Differentiable form: hand-written reverse of si_euler steps with the
 * neighbour list frozen per step, the way the reference differentiates a
 * rollout with jax.grad(..., allow_int=True) (notebooks/iclr24_grads.ipynb,
 * notebooks/iclr24_inverse.ipynb). Covers one case of the SPH solver with
 * density summation, any transport-velocity factor, optionally the no-slip
 * generalized wall BC (no external force then) with a velocity bc_fn, and no
 * artificial viscosity. sph_adjoint_init allocates a tape of `slots` steps.
 * sph_tape_record saves the forward data of the step just taken by sph_step
 * into a slot. sph_adjoint_step maps, in place, the adjoints of a recorded
 * step's outputs r, u, dudt, dvdt (lam_r, lam_u, lam_a, lam_b) to those of its
 * inputs. Adjoint arrays are (n, dim) float32 device arrays in the original
 * particle order. */
int sph_adjoint_init(SphHandle* h, int32_t slots);
int sph_tape_record(SphHandle* h, int32_t slot, void* stream);
int sph_adjoint_step(SphHandle* h, int32_t slot, float* lam_r, float* lam_u, float* lam_a,
                     float* lam_b, void* stream);
/* A checkpoint segment in one call each way. sph_tape_segment runs `nsteps`
 * steps like sph_step from the loaded state, recording step t into slot t
 * (nsteps <= slots). sph_adjoint_segment then applies sph_adjoint_step to
 * slots nsteps-1 down to 0. */
int sph_tape_segment(SphHandle* h, int32_t nsteps, void* stream);
/* Device snapshots of a handle's state between two steps, for the
 * differentiable form's checkpoints: sph_snapshot_init allocates `slots`
 * snapshots (the resident particle set, the pending forward result, the
 * binning and the candidate lists: ~0.5 KB per particle each);
 * sph_snapshot_save copies the state after an sph_step into a slot and
 * sph_snapshot_restore copies it back, so that the following steps repeat
 * the saved ones bit for bit (including the order in which pairs are summed)
 * without re-binning. SPH solver with density summation, no heat conduction.
 * Replaces the reference's in-memory JAX tape (notebooks/iclr24_grads.ipynb):
 * no counterpart of its own. */
int sph_snapshot_init(SphHandle* h, int32_t slots);
int sph_snapshot_save(SphHandle* h, int32_t slot, void* stream);
int sph_snapshot_restore(SphHandle* h, int32_t slot, void* stream);
int sph_adjoint_segment(SphHandle* h, int32_t nsteps, float* lam_r, float* lam_u, float* lam_a,
                        float* lam_b, void* stream);

/* Read (and optionally clear) the device status word. Synchronizes `stream`.
 * sph_set_state clears the word. */
int sph_read_status(SphHandle* h, uint32_t* status, int32_t clear, void* stream);
/* Stream-ordered copy of the device status word into `status_dev` (a device
 * uint32), optionally clearing it; no host synchronization. The way the
 * reference keeps NeighborList.error as a device value until the caller
 * tests it (jax_md/partition.py:460-499). */
int sph_read_status_async(SphHandle* h, uint32_t* status_dev, int32_t clear, void* stream);

/* Allocation-free neighbour list (no counterpart in the reference: it exists
 * for callers that cannot call cudaMalloc, such as a host framework that owns
 * the whole device memory pool, or code that must not allocate after start-up).
 * Same edges, order and padding as sph_nl_edges for `n` positions r (device,
 * (n, dim) float32) in a periodic box with the reference's cutoff test; no
 * handle and no allocation: all scratch lives in one fixed file-scope device
 * array of about 4 MB, so n <= SPH_NOALLOC_MAX_PARTICLES and the cell grid
 * must have <= SPH_NOALLOC_MAX_CELLS cells (larger inputs are rejected with
 * SPH_ERR_INVALID_ARG before any GPU work). The array is shared by all calls
 * on a device: calls that overlap on the GPU race and must be ordered by the
 * caller. The first call on a device looks up the array's address
 * (cudaGetSymbolAddress, with that device current) and should come before any
 * stream capture. The looked-up address is kept for the life of the process:
 * do not reset the device (cudaDeviceReset) between calls. Cost: the sort
 * ranks each particle within its cell and the emission sorts each sender's
 * receivers by insertion, so both grow with the square of the occupancy of
 * a cell or of a neighbourhood; inputs that pile many particles into one cell
 * (thousands, far beyond an SPH particle spacing) make a call slow.
 * *count_dev receives the edge count; *status_dev (optional, device) the
 * call's status bits. */
#define SPH_NOALLOC_MAX_PARTICLES 65536
#define SPH_NOALLOC_MAX_CELLS 65536
int sph_nl_edges_noalloc(int32_t dim, const double* box, double r_cutoff, int32_t mask_self,
                         const float* r, int64_t n, int32_t* idx, int64_t capacity,
                         int64_t* count_dev, uint32_t* status_dev, void* stream);

/* Float64 global diagnostics per case, computed on the GPU in double
 * precision: out[c*8 + k] = {mass, mom_x, mom_y, mom_z, E_kin, u_max, rho_min,
 * rho_max} of case c (fluid particles; E_kin follows jax_sph/utils.py:128-133).
 * `out` is a device array of n_cases*8 doubles. */
int sph_diagnostics(SphHandle* h, double* out, void* stream);
/* Per-particle size of the neighbour set the last forward pass (sph_forward,
 * sph_step, sph_advance) summed over: counts[i] (original order, device
 * int32 array of n) = the number of edges whose receiver is particle i, self
 * pair included unless mask_self -- i.e. the number of entries of i in row 0
 * of the reference's NeighborList.idx for the same positions
 * (jax_md/partition.py:885-909). No counterpart function in the reference; a
 * diagnostic of the per-step sets. */
int sph_neighbour_counts(SphHandle* h, int32_t* counts, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SPH_GB300_H */
