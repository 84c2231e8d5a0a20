"""Equations of state (``jax_sph/eos.py:20-57``).

The parameters are handed to the CUDA kernels (``eos_p``/``eos_rho`` in
``csrc/sph_internal.cuh``); ``p_fn``/``rho_fn`` evaluate the same formulas on
tensors or floats.
"""


class TaitEoS:
    """Tait EOS ``p = p_ref((rho/rho_ref)^gamma - 1) + p_bg`` (eos.py:20-38)."""

    kind = 0

    def __init__(self, p_ref, rho_ref, p_background, gamma):
        self.p_ref = p_ref
        self.rho_ref = rho_ref
        self.p_bg = p_background
        self.gamma = gamma
        self.u_ref = 1.0

    def p_fn(self, rho):
        return self.p_ref * ((rho / self.rho_ref) ** self.gamma - 1) + self.p_bg

    def rho_fn(self, p):
        p_temp = p + self.p_ref - self.p_bg
        return self.rho_ref * (p_temp / self.p_ref) ** (1 / self.gamma)


class RIEMANNEoS:
    """Riemann-SPH EOS ``p = 100 u_ref^2 (rho - rho_ref) + p_bg`` (eos.py:41-57)."""

    kind = 1

    def __init__(self, rho_ref, p_background, u_ref):
        self.rho_ref = rho_ref
        self.u_ref = u_ref
        self.p_bg = p_background
        self.p_ref = 100 * u_ref ** 2 * rho_ref
        self.gamma = 1.0

    def p_fn(self, rho):
        return 100 * self.u_ref ** 2 * (rho - self.rho_ref) + self.p_bg

    def rho_fn(self, p):
        return (p - self.p_bg) / (100 * self.u_ref ** 2) + self.rho_ref
