"""ctypes binding of ``libsph_gb300.so`` and the ``Engine`` handle wrapper.

This is the Python side of the C ABI in ``include/sph_gb300.h``. There is no
fallback: if the shared library cannot be loaded, or no CUDA device is
present, every call raises.
"""

import ctypes
import os

import numpy as np
import torch

from . import _build

# status bits (include/sph_gb300.h)
NEIGHBOR_LIST_OVERFLOW = 0x1
CELL_LIST_OVERFLOW = 0x2
CELL_SIZE_TOO_SMALL = 0x4
MALFORMED_BOX = 0x8
ERR_INVALID_ARG = 0x100
ERR_CUDA = 0x200
ERR_TIMEOUT = 0x400
ERR_NONFINITE = 0x800
INFO_MOVED = 0x2000
WARN_BOX_EDGE = 0x1000
ERR_HOST = 0x4000

KERNELS = {"QSK": 0, "WC2K": 1}
SOLVERS = {"SPH": 0, "RIE": 1, "DELTA": 2}
EOS_TAIT, EOS_RIEMANN = 0, 1
GEXT_ZERO, GEXT_CONST, GEXT_BAND_X, GEXT_ARRAY, GEXT_REVERSE_X = 0, 1, 2, 3, 4
FORCE_GATHER, FORCE_STAGED = 0, 1
BC_NONE, BC_SOLID_ZERO, BC_SOLID_ZERO_P, BC_LID, BC_HT = 0, 1, 2, 3, 4
NL_JAXMD, NL_MATSCIPY = 0, 1
TAG_PAD = -1  # Tag.PAD_VALUE (utils.py:25)


class SphConfig(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("kernel", ctypes.c_int32), ("solver", ctypes.c_int32),
                ("is_rho_evol", ctypes.c_int32), ("is_bc_trick", ctypes.c_int32),
                ("is_free_slip", ctypes.c_int32), ("mask_self", ctypes.c_int32),
                ("kahan", ctypes.c_int32), ("fp64_positions", ctypes.c_int32),
                ("capacity_multiplier", ctypes.c_double), ("verlet_skin", ctypes.c_double),
                ("canonical_order", ctypes.c_int32), ("is_rho_renorm", ctypes.c_int32),
                ("is_heat_conduction", ctypes.c_int32), ("nl_backend", ctypes.c_int32)]


class SphCase(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("box", ctypes.c_double * 3), ("r_cutoff", ctypes.c_double),
                ("dx", ctypes.c_double), ("h", ctypes.c_double), ("dt", ctypes.c_double),
                ("dt_solver", ctypes.c_double), ("tvf", ctypes.c_double),
                ("c_ref", ctypes.c_double), ("eos", ctypes.c_int32), ("g_kind", ctypes.c_int32),
                ("bc_kind", ctypes.c_int32), ("pad0", ctypes.c_int32),
                ("p_ref", ctypes.c_double), ("rho_ref", ctypes.c_double),
                ("p_bg", ctypes.c_double), ("gamma", ctypes.c_double),
                ("u_ref", ctypes.c_double), ("eta_limiter", ctypes.c_double),
                ("artificial_alpha", ctypes.c_double), ("g", ctypes.c_double * 3),
                ("g_band_lo", ctypes.c_double), ("g_band_hi", ctypes.c_double),
                ("u_lid", ctypes.c_double * 3), ("diff_alpha", ctypes.c_double),
                ("diff_delta", ctypes.c_double), ("bc_T", ctypes.c_double * 2),
                ("bc_x", ctypes.c_double * 2)]


class SphStateView(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64)] + [
        (k, ctypes.c_void_p) for k in ("r", "tag", "u", "v", "dudt", "dvdt", "drhodt", "rho",
                                       "p", "mass", "eta", "nw", "g_ext", "T", "dTdt",
                                       "kappa", "Cp")]


class SphNLCapacity(ctypes.Structure):
    _fields_ = [("cell_capacity", ctypes.c_int64), ("max_occupancy", ctypes.c_int64),
                ("occupancy", ctypes.c_int64), ("max_cell_occupancy", ctypes.c_int64)]


EXPORTS = ["sph_abi_version", "sph_last_error", "sph_create", "sph_destroy", "sph_update_cases",
           "sph_set_state", "sph_get_state", "sph_nl_allocate", "sph_nl_set_capacity",
           "sph_nl_update", "sph_nl_edges", "sph_forward", "sph_step", "sph_set_block_size",
           "sph_set_force_variant",
           "sph_step_launch_count", "sph_profile_step", "sph_adjoint_init", "sph_tape_record",
           "sph_adjoint_step", "sph_read_status", "sph_read_status_async", "sph_diagnostics",
           "sph_nl_edges_noalloc", "sph_rebuild_stats", "sph_advance", "sph_set_wall_layer",
           "sph_neighbour_counts", "sph_tape_segment", "sph_adjoint_segment",
           "sph_list_format", "sph_snapshot_init", "sph_snapshot_save", "sph_snapshot_restore"]

_LIB = None


def load(build_if_missing=True):
    """Load (building if needed) the shared library and declare its signatures."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing; run the build first")
        _build.build()
    lib = ctypes.CDLL(path)
    P, I, V = ctypes.POINTER, ctypes.c_int, ctypes.c_void_p
    lib.sph_abi_version.restype = I
    lib.sph_last_error.restype = ctypes.c_char_p
    lib.sph_create.argtypes = [P(SphConfig), P(SphCase), ctypes.c_int32, P(V)]
    lib.sph_destroy.argtypes = [V]
    lib.sph_update_cases.argtypes = [V, P(SphCase), ctypes.c_int32]
    lib.sph_set_state.argtypes = [V, P(SphStateView), V]
    lib.sph_get_state.argtypes = [V, P(SphStateView), V]
    lib.sph_nl_allocate.argtypes = [V, ctypes.c_int64, P(SphNLCapacity), V]
    lib.sph_nl_set_capacity.argtypes = [V, P(SphNLCapacity)]
    lib.sph_nl_update.argtypes = [V, V]
    lib.sph_nl_edges.argtypes = [V, V, ctypes.c_int64, V, V]
    lib.sph_forward.argtypes = [V, V]
    lib.sph_step.argtypes = [V, ctypes.c_int32, V]
    lib.sph_set_block_size.argtypes = [V, ctypes.c_int32]
    lib.sph_set_force_variant.argtypes = [V, ctypes.c_int32]
    lib.sph_step_launch_count.argtypes = [V, P(ctypes.c_int32)]
    lib.sph_list_format.argtypes = [V, P(ctypes.c_int32)]
    lib.sph_snapshot_init.argtypes = [V, ctypes.c_int32]
    lib.sph_snapshot_save.argtypes = [V, ctypes.c_int32, V]
    lib.sph_snapshot_restore.argtypes = [V, ctypes.c_int32, V]
    lib.sph_profile_step.argtypes = [V, ctypes.c_int32, P(ctypes.c_float), V]
    lib.sph_adjoint_init.argtypes = [V, ctypes.c_int32]
    lib.sph_tape_record.argtypes = [V, ctypes.c_int32, V]
    lib.sph_adjoint_step.argtypes = [V, ctypes.c_int32, V, V, V, V, V]
    lib.sph_read_status.argtypes = [V, P(ctypes.c_uint32), ctypes.c_int32, V]
    lib.sph_read_status_async.argtypes = [V, V, ctypes.c_int32, V]
    lib.sph_rebuild_stats.argtypes = [V, P(ctypes.c_int64), P(ctypes.c_int32), V]
    lib.sph_advance.argtypes = [V, P(SphStateView), P(SphStateView), V, ctypes.c_float, V, V]
    lib.sph_neighbour_counts.argtypes = [V, V, V]
    lib.sph_tape_segment.argtypes = [V, ctypes.c_int32, V]
    lib.sph_adjoint_segment.argtypes = [V, ctypes.c_int32, V, V, V, V, V]
    lib.sph_diagnostics.argtypes = [V, V, V]
    lib.sph_set_wall_layer.argtypes = [V, V, ctypes.c_int64, P(ctypes.c_double), ctypes.c_double]
    lib.sph_nl_edges_noalloc.argtypes = [ctypes.c_int32, P(ctypes.c_double), ctypes.c_double,
                                         ctypes.c_int32, V, ctypes.c_int64, V, ctypes.c_int64,
                                         V, V, V]
    for name in EXPORTS:
        if name not in ("sph_abi_version", "sph_last_error"):
            getattr(lib, name).restype = I
    if lib.sph_abi_version() != 7:
        raise RuntimeError("libsph_gb300 ABI version mismatch")
    _LIB = lib
    return lib


class SphError(RuntimeError):
    """A failing C-ABI call (the message comes from ``sph_last_error``)."""

    def __init__(self, code, msg):
        super().__init__(f"{msg} (status 0x{code:x})")
        self.code = code


def _check(rc):
    if rc != 0:
        raise SphError(rc, _LIB.sph_last_error().decode())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


_VEC_OUT = ("r", "u", "v", "dudt", "dvdt", "nw")


def host_outputs(n, dim, keys):
    """Result arrays of a drop-in step in ONE pinned host block (one
    allocation per step): a dict of float32 tensors (``(n, dim)`` for vector
    fields, ``(n,)`` for scalars), a one-element int32 status word in the
    same block and the ``SphStateView`` over the arrays. The vector fields
    come first, then the scalars (each group one ``unbind``)."""
    vec = [k for k in keys if k in _VEC_OUT]
    sca = [k for k in keys if k not in _VEC_OUT]
    nv, ns = len(vec) * n * dim, len(sca) * n
    flat = torch.empty(nv + ns + 4, dtype=torch.float32, pin_memory=True)
    out = dict(zip(vec, flat[:nv].view(len(vec), n, dim).unbind(0)))
    out.update(zip(sca, flat[nv:nv + ns].view(len(sca), n).unbind(0)))
    status = flat[nv + ns:nv + ns + 1].view(torch.int32)
    base = flat.data_ptr()
    v = SphStateView()
    v.n = n
    for i, k in enumerate(vec):
        setattr(v, k, base + 4 * i * n * dim)
    for i, k in enumerate(sca):
        setattr(v, k, base + 4 * (nv + i * n))
    return out, status, v


try:
    _raw_stream_of = torch._C._cuda_getCurrentRawStream
except AttributeError:  # pragma: no cover - older builds
    _raw_stream_of = None


def raw_stream():
    """The current CUDA stream as a raw handle (the cheap way where torch has it)."""
    if _raw_stream_of is not None:
        return _raw_stream_of(torch.cuda.current_device())
    return torch.cuda.current_stream().cuda_stream


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("jaxsph_gb300 needs a CUDA device (GB300, sm_103a); none is available")


class Engine:
    """Owner of one ``SphHandle``: a set of cases with one configuration."""

    def __init__(self, config: SphConfig, cases):
        require_cuda()
        self.lib = load()
        self.config = config
        self.cases = list(cases)
        self.n = sum(int(c.n) for c in self.cases)
        arr = (SphCase * len(self.cases))(*self.cases)
        h = ctypes.c_void_p()
        _check(self.lib.sph_create(ctypes.byref(config), arr, len(self.cases), ctypes.byref(h)))
        self.h = h
        self._keep = None  # tensors referenced by the last SphStateView

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value and _LIB is not None:
            _LIB.sph_destroy(h)
            self.h = None

    def update_cases(self, cases):
        cases = list(cases)
        arr = (SphCase * len(cases))(*cases)
        _check(self.lib.sph_update_cases(self.h, arr, len(cases)))
        self.cases = cases

    @staticmethod
    def view(state, n, pinned_ok=False):
        """SphStateView over a dict of contiguous float32/int32 CUDA tensors
        (or pinned host tensors, where ``pinned_ok``)."""
        v = SphStateView()
        v.n = n
        for k in ("r", "tag", "u", "v", "dudt", "dvdt", "drhodt", "rho", "p", "mass", "eta",
                  "nw", "g_ext", "T", "dTdt", "kappa", "Cp"):
            t = state.get(k)
            if t is not None:
                # host tensors: the library itself refuses pageable memory
                ok = t.is_cuda or (pinned_ok and t.device.type == "cpu")
                if not ok or not t.is_contiguous():
                    raise ValueError(f"state['{k}'] must be a contiguous CUDA tensor"
                                     + (" or pinned host tensor" if pinned_ok else ""))
                want = torch.int32 if k == "tag" else torch.float32
                if t.dtype != want:
                    raise ValueError(f"state['{k}'] must be {want}, got {t.dtype}")
                setattr(v, k, t.data_ptr())
        return v

    def set_state(self, state):
        v = self.view(state, self.n)
        self._keep = state
        _check(self.lib.sph_set_state(self.h, ctypes.byref(v), _stream()))

    def get_state(self, out):
        v = self.view(out, self.n)
        _check(self.lib.sph_get_state(self.h, ctypes.byref(v), _stream()))

    def nl_allocate(self, extra_capacity=0):
        cap = SphNLCapacity()
        _check(self.lib.sph_nl_allocate(self.h, int(extra_capacity), ctypes.byref(cap), _stream()))
        return cap

    def nl_set_capacity(self, cell_capacity, max_occupancy):
        cap = SphNLCapacity(int(cell_capacity), int(max_occupancy), 0, 0)
        _check(self.lib.sph_nl_set_capacity(self.h, ctypes.byref(cap)))

    def nl_update(self):
        _check(self.lib.sph_nl_update(self.h, _stream()))

    def nl_edges(self, capacity, device):
        idx = torch.empty((2, int(capacity)), dtype=torch.int32, device=device)
        count = torch.zeros(1, dtype=torch.int64, device=device)
        _check(self.lib.sph_nl_edges(self.h, _ptr(idx), int(capacity), _ptr(count), _stream()))
        return idx, count

    def forward(self):
        _check(self.lib.sph_forward(self.h, _stream()))

    def step(self, nsteps=1):
        _check(self.lib.sph_step(self.h, int(nsteps), _stream()))

    def set_block_size(self, threads):
        _check(self.lib.sph_set_block_size(self.h, int(threads)))

    def set_force_variant(self, variant):
        """FORCE_GATHER or FORCE_STAGED: how the lean force pass reads its
        senders (the same results either way)."""
        _check(self.lib.sph_set_force_variant(self.h, int(variant)))

    def launch_count(self):
        c = ctypes.c_int32(0)
        _check(self.lib.sph_step_launch_count(self.h, ctypes.byref(c)))
        return int(c.value)

    def snapshot_init(self, slots):
        _check(self.lib.sph_snapshot_init(self.h, int(slots)))

    def snapshot_save(self, slot):
        """Copy the state between two steps into device snapshot ``slot``."""
        _check(self.lib.sph_snapshot_save(self.h, int(slot), _stream()))

    def snapshot_restore(self, slot):
        """Copy snapshot ``slot`` back: the next steps repeat the saved ones bit for bit."""
        _check(self.lib.sph_snapshot_restore(self.h, int(slot), _stream()))

    def list_format(self):
        """0: generic passes; 1 / 2: lean passes with 16-bit / 32-bit lists."""
        f = ctypes.c_int32(0)
        _check(self.lib.sph_list_format(self.h, ctypes.byref(f)))
        return int(f.value)

    def profile(self, nsteps, split=False):
        """Average per-step milliseconds of (kick + rebuilds, density, wall,
        force); with ``split`` also (kick alone, rebuilds alone)."""
        ms = (ctypes.c_float * 6)()
        _check(self.lib.sph_profile_step(self.h, int(nsteps), ms, _stream()))
        out = [float(x) for x in ms]
        return out if split else out[:4]

    def adjoint_init(self, slots):
        _check(self.lib.sph_adjoint_init(self.h, int(slots)))

    def tape_segment(self, nsteps):
        """Run ``nsteps`` steps, recording step t into tape slot t."""
        _check(self.lib.sph_tape_segment(self.h, int(nsteps), _stream()))

    def adjoint_segment(self, nsteps, lam_r, lam_u, lam_a, lam_b):
        """Reverse slots nsteps-1 .. 0, all four adjoints in place."""
        self._adjoint_arrays(lam_r, lam_u, lam_a, lam_b)
        _check(self.lib.sph_adjoint_segment(self.h, int(nsteps), _ptr(lam_r), _ptr(lam_u),
                                            _ptr(lam_a), _ptr(lam_b), _stream()))

    def tape_record(self, slot):
        _check(self.lib.sph_tape_record(self.h, int(slot), _stream()))

    @staticmethod
    def _adjoint_arrays(*ts):
        for t in ts:
            if not (t.is_cuda and t.is_contiguous() and t.dtype == torch.float32):
                raise ValueError("adjoint arrays must be contiguous float32 CUDA tensors")

    def adjoint_step(self, slot, lam_r, lam_u, lam_a, lam_b):
        """Reverse one recorded step, all four adjoints in place."""
        self._adjoint_arrays(lam_r, lam_u, lam_a, lam_b)
        _check(self.lib.sph_adjoint_step(self.h, int(slot), _ptr(lam_r), _ptr(lam_u),
                                         _ptr(lam_a), _ptr(lam_b), _stream()))

    def set_wall_layer(self, layer, offset, cutoff):
        """Recompute the wall normals every step from a static fine wall layer
        (host ``(m, dim)`` float32 array; ``None`` switches it off)."""
        if layer is None:
            _check(self.lib.sph_set_wall_layer(self.h, None, 0, None, 0.0))
            return
        arr = np.ascontiguousarray(np.asarray(layer, dtype=np.float32))
        off = (ctypes.c_double * 3)(*[float(x) for x in list(offset) + [0.0] * (3 - len(offset))])
        _check(self.lib.sph_set_wall_layer(self.h, arr.ctypes.data, int(arr.shape[0]), off,
                                           float(cutoff)))

    def read_status(self, clear=False):
        s = ctypes.c_uint32(0)
        _check(self.lib.sph_read_status(self.h, ctypes.byref(s), int(bool(clear)), _stream()))
        return int(s.value)

    def advance(self, state, out, ref=None, threshold_sq=0.0, vin=None, vout=None,
                status=None, stream=None):
        """One fused drop-in step (load, step, read back); returns the status
        word, by default a 0-d int32 device tensor (no host synchronisation).
        ``vin`` / ``vout``: views of ``state`` / ``out`` already built (see
        ``next_view`` and ``host_outputs``); ``status``: where the word goes
        (a device or pinned host int32 tensor); ``stream``: a raw stream
        handle (default: the current stream). With any result in host memory
        the call returns once it is there."""
        vin = vin if vin is not None else self.view(state, self.n, pinned_ok=True)
        vout = vout if vout is not None else self.view(out, self.n, pinned_ok=True)
        self._views = (vin, vout)
        if status is None:
            status = torch.empty((), dtype=torch.int32, device="cuda")
        self._keep = state
        _check(self.lib.sph_advance(self.h, ctypes.byref(vin), ctypes.byref(vout),
                                    _ptr(ref) if ref is not None else None,
                                    float(threshold_sq), status.data_ptr(),
                                    stream if stream is not None else raw_stream()))
        return status

    def next_view(self):
        """The input view of a state made of the last advance's outputs and its
        inputs' other fields (tag, mass, eta, nw, g_ext)."""
        vin, vout = self._views
        v = SphStateView.from_buffer_copy(vin)
        for k in ("r", "u", "v", "dudt", "dvdt", "drhodt", "rho", "p", "T", "dTdt", "nw"):
            if getattr(vout, k):  # a field not written is the input's own
                setattr(v, k, getattr(vout, k))
        return v

    def rebuild_stats(self):
        """(candidate-list rebuilds so far, kernels per rebuild); synchronises."""
        n, k = ctypes.c_int64(0), ctypes.c_int32(0)
        _check(self.lib.sph_rebuild_stats(self.h, ctypes.byref(n), ctypes.byref(k), _stream()))
        return int(n.value), int(k.value)

    def read_status_async(self, clear=False):
        """The status word as a 0-d int32 device tensor (stream-ordered, no sync)."""
        out = torch.empty((), dtype=torch.int32, device="cuda")
        _check(self.lib.sph_read_status_async(self.h, _ptr(out), int(bool(clear)), _stream()))
        return out

    def neighbour_counts(self, device):
        """Per particle (original order) the size of its neighbour set in the
        last forward pass, self pair included unless masked (int32 device tensor)."""
        out = torch.empty(self.n, dtype=torch.int32, device=device)
        _check(self.lib.sph_neighbour_counts(self.h, _ptr(out), _stream()))
        return out

    def diagnostics(self, device):
        out = torch.empty((len(self.cases), 8), dtype=torch.float64, device=device)
        _check(self.lib.sph_diagnostics(self.h, _ptr(out), _stream()))
        return out
