"""Per-instance algorithm choice for batches.

Three dispatchers share one interface (`choose(specs) -> [ndconv_algo]`):
  * ModelDispatcher: the library's cost model (ndconv_plan_info): direct (0)
    or FFT (1, form picked inside the library);
  * TunedDispatcher: the autotuner's timing database (measured, exhaustive);
  * MLPDispatcher (ndconv.mlp): the network trained on those timings."""
import ctypes
import math

import numpy as np

from . import _abi
from .api import build_problem, into_kernel_with_dilation

N_FEATURES = 16


def plan_info(problem):
    out = (ctypes.c_double * 8)()
    st = _abi.lib().ndconv_plan_info(ctypes.byref(problem), out)
    if st:
        raise RuntimeError(_abi.last_error())
    return list(out)


def spec_problem(spec, dtype=_abi.F32):
    import numpy as _np
    k = _np.zeros(spec.kshape, dtype=_np.float32)
    from .api import with_dilation
    return build_problem(dtype, spec.shape, with_dilation(k, spec.dilation), spec.conv_mode(),
                         spec.padding_mode())


def features(spec):
    """16 shape / mode features (log-scaled) of one instance."""
    r = spec.rank
    sh = list(spec.shape) + [1] * (3 - r)
    ks = list(spec.kshape) + [1] * (3 - r)
    info = plan_info(spec_problem(spec))
    pad = {"Zeros": 0, "Reflect": 1, "Replicate": 2, "Circular": 3}[spec.pad]
    f = [math.log2(s) for s in sh] + [math.log2(k) for k in ks]
    f += [float(r), float(spec.dilation), float(spec.stride), float(pad)]
    f += [math.log2(max(info[2], 1.0)), math.log2(max(info[3], 1.0)),
          math.log2(max(info[4] * info[5] * info[6], 1.0)), float(info[7]),
          math.log2(max(info[0], 1e-9)) - math.log2(max(min(info[1], 1e9), 1e-9))]
    f += [0.0]  # dtype f32
    assert len(f) == N_FEATURES
    return f


class ModelDispatcher:
    """argmin of the library's modelled times."""

    def choose(self, specs):
        out = []
        for s in specs:
            info = plan_info(spec_problem(s))
            out.append(1 if info[7] and info[1] < info[0] else 0)
        return out


class TunedDispatcher:
    """argmin of measured times from the autotuner's database (the cost
    model for instances it has not timed)."""

    def __init__(self, db):
        self.db = db

    def choose(self, specs):
        from .autotune import MEASURED
        out = []
        for s in specs:
            t = self.db.lookup(s)
            if t is None:
                info = plan_info(spec_problem(s))
                out.append(1 if info[7] and info[1] < info[0] else 0)
            else:
                out.append(int(MEASURED[int(np.argmin(t[:6]))]))
        return out
