"""SPH interpolation kernels on the hot path (``jax_sph/kernel.py:51-103``).

The CUDA kernels evaluate W and dW/dr in float32 (``kw``/``kdw`` in
``csrc/sph_internal.cuh``); these classes carry the parameters (cutoff,
normalisation) the engine needs and give tensor evaluations of the same
closed forms for user-side work. The reference obtains ``grad_w`` by autodiff
of ``w`` (kernel.py:20-23); here it is the analytic derivative.
"""

import math

import torch


class QuinticKernel:
    """Morris quintic spline, cutoff 3h (kernel.py:51-72)."""

    name = "QSK"

    def __init__(self, h, dim=3):
        self.h = h
        self.dim = dim
        self._one_over_h = 1.0 / h
        self._normalized_cutoff = 3.0
        self.cutoff = self._normalized_cutoff * h
        self._sigma = {1: 1.0 / 120.0 * self._one_over_h,
                       2: 7.0 / 478.0 / math.pi * self._one_over_h ** 2,
                       3: 3.0 / 359.0 / math.pi * self._one_over_h ** 3}[dim]

    def w(self, r):
        q = r * self._one_over_h
        q1 = torch.clamp(1.0 - q, min=0.0)
        q2 = torch.clamp(2.0 - q, min=0.0)
        q3 = torch.clamp(3.0 - q, min=0.0)
        return self._sigma * (q3 ** 5 - 6.0 * q2 ** 5 + 15.0 * q1 ** 5)

    def grad_w(self, r):
        q = r * self._one_over_h
        q1 = torch.clamp(1.0 - q, min=0.0)
        q2 = torch.clamp(2.0 - q, min=0.0)
        q3 = torch.clamp(3.0 - q, min=0.0)
        return -5.0 * self._sigma * self._one_over_h * (q3 ** 4 - 6.0 * q2 ** 4 + 15.0 * q1 ** 4)


class WendlandC2Kernel:
    """Wendland C2, cutoff 2h (kernel.py:75-103)."""

    name = "WC2K"

    def __init__(self, h, dim=3):
        self.h = h
        self.dim = dim
        self._one_over_h = 1.0 / h
        self._normalized_cutoff = 2.0
        self.cutoff = self._normalized_cutoff * h
        self._sigma = {1: 5.0 / 8.0 * self._one_over_h,
                       2: 7.0 / 4.0 / math.pi * self._one_over_h ** 2,
                       3: 21.0 / 16.0 / math.pi * self._one_over_h ** 3}[dim]

    def w(self, r):
        q = r * self._one_over_h
        q1 = torch.clamp(1.0 - 0.5 * q, min=0.0)
        if self.dim == 1:
            return self._sigma * q1 ** 3 * (1.5 * q + 1.0)
        return self._sigma * q1 ** 4 * (2.0 * q + 1.0)

    def grad_w(self, r):
        q = r * self._one_over_h
        q1 = torch.clamp(1.0 - 0.5 * q, min=0.0)
        if self.dim == 1:
            return self._sigma * self._one_over_h * (-1.5 * q1 ** 2 * (1.5 * q + 1.0) + 1.5 * q1 ** 3)
        return -5.0 * self._sigma * self._one_over_h * q * q1 ** 3


KERNELS = {"QSK": QuinticKernel, "WC2K": WendlandC2Kernel}


def make_kernel(name, h, dim):
    if name not in KERNELS:
        raise NotImplementedError(
            f"kernel {name!r}: only the hot-path kernels QSK and WC2K are implemented")
    return KERNELS[name](h=h, dim=dim)
