"""Seeded synthetic workloads (no public dataset is involved).

uneven_batch: the uneven batch of instances used by the batch benchmark and
the dispatcher's training set: rank drawn from {1: 60%, 2: 35%, 3: 5%},
total input elements log-uniform in [2^8, 2^20] split across axes by
Dirichlet proportions of the log size, odd kernel extents uniform in 3..127
per axis, dilation in {1, 2}, stride in {1, 2}, padding mode uniform over
Zeros / Reflect / Replicate / Circular, f32 values Uniform[-1, 1).  The
conv mode is Explicit with Same's pads and the drawn strides (Same itself
forces stride 1).
"""
import math

import numpy as np

from .api import ConvMode, PaddingMode

PAD_MODES = ("Zeros", "Reflect", "Replicate", "Circular")


class Spec:
    __slots__ = ("shape", "kshape", "dilation", "stride", "pad", "rank")

    def __init__(self, shape, kshape, dilation, stride, pad):
        self.shape, self.kshape = tuple(shape), tuple(kshape)
        self.dilation, self.stride, self.pad = dilation, stride, pad
        self.rank = len(shape)

    def keff(self):
        return [k * self.dilation - self.dilation + 1 for k in self.kshape]

    def conv_mode(self):
        pads = [[(e - 1) // 2, (e - 1) // 2] for e in self.keff()]  # odd extents
        return ConvMode.Explicit(pads, [self.stride] * self.rank)

    def padding_mode(self):
        return getattr(PaddingMode, self.pad)

    def out_shape(self):
        return [(n + e - 1 - e) // self.stride + 1 for n, e in zip(self.shape, self.keff())]

    def bytes(self):
        """algorithmic bytes 4 (|x| + |k| + |y|)"""
        return 4 * (math.prod(self.shape) + math.prod(self.kshape) + math.prod(self.out_shape()))

    def __repr__(self):
        return (f"Spec(shape={self.shape}, kernel={self.kshape}, dil={self.dilation}, "
                f"stride={self.stride}, pad={self.pad})")


def uneven_batch(n=4096, seed=0, min_log2=8, max_log2=20, kmin=3, kmax=127,
                 rank_p=(0.6, 0.35, 0.05), max_axis=None, kmax_2d=None):
    rng = np.random.default_rng(seed)
    out = []
    odd = np.arange(kmin | 1, kmax + 1, 2)
    for _ in range(n):
        rank = int(rng.choice([1, 2, 3], p=rank_p))
        total = math.exp(rng.uniform(min_log2 * math.log(2), max_log2 * math.log(2)))
        props = rng.dirichlet(np.ones(rank))
        shape = [max(1, int(round(total ** p))) for p in props]
        if max_axis:
            shape = [min(s, max_axis) for s in shape]
        ks = odd if (kmax_2d is None or rank < 2) else odd[odd <= kmax_2d]
        kshape = [int(rng.choice(ks)) for _ in range(rank)]
        dil = int(rng.choice([1, 2]))
        stride = int(rng.choice([1, 2]))
        pad = PAD_MODES[int(rng.integers(0, 4))]
        out.append(Spec(shape, kshape, dil, stride, pad))
    return out


def make_tensors(specs, seed=0, device="cuda"):
    """Seeded Uniform[-1, 1) f32 data and kernels for the specs."""
    import torch
    g = torch.Generator(device=device).manual_seed(seed)
    xs = [torch.rand(s.shape, generator=g, device=device) * 2 - 1 for s in specs]
    ks = [torch.rand(s.kshape, generator=g, device=device) * 2 - 1 for s in specs]
    return xs, ks
