"""Heterogeneous batches: many independent convolutions in one submission.

BatchPlan binds n problems (any shapes, kernels, modes; f32 ones run inside
one persistent kernel with a device work queue, replayed as a CUDA graph)
to their device buffers.  `algos[i]` picks the variant (ndconv_algo: direct 0,
FFT 1, FFT plan variants 3..6) per
instance; `ndconv.dispatch` chooses them by cost model, timing DB or MLP.
"""
import ctypes

import torch

from . import _abi
from .api import KernelWithDilation, build_problem, dtype_code, into_kernel_with_dilation

INFO_FIELDS = ("tasks", "grid", "smem", "n_fft", "n_direct", "n_standalone", "workspace_bytes", "counters")


class BatchPlan:
    def __init__(self, specs, datas, kernels, outs=None, algos=None):
        """specs: list of (conv_mode, padding_mode); datas / kernels: CUDA
        tensors (kernels may be KernelWithDilation); outs: preallocated
        outputs or None (allocated here)."""
        L = _abi.lib()
        n = len(datas)
        self.n = n
        self.datas = [d.contiguous() for d in datas]
        kws = [into_kernel_with_dilation(k) for k in kernels]
        self.kernels = [k.kernel.contiguous() for k in kws]
        probs = (_abi.Problem * max(n, 1))()
        self.problems = probs
        shape = (ctypes.c_int64 * 3)()
        self.outs = []
        for i in range(n):
            cm, pm = specs[i]
            kw = KernelWithDilation(self.kernels[i], kws[i].dilation, kws[i].reverse_flag)
            p = build_problem(dtype_code(self.datas[i].dtype), tuple(self.datas[i].shape), kw, cm, pm)
            probs[i] = p
            algo = 1 if algos is None else int(algos[i])
            # output_shape knows the two argument-check orders: direct (0) and FFT (1)
            st = L.ndconv_output_shape(ctypes.byref(p), 0 if algo in (0, 2) else 1, shape)
            if st:
                raise RuntimeError(f"instance {i}: {_abi.last_error()}")
            if outs is None:
                self.outs.append(torch.empty([shape[j] for j in range(p.rank)], dtype=self.datas[i].dtype,
                                             device=self.datas[i].device))
            else:
                self.outs.append(outs[i])
        self.algos = (ctypes.c_int32 * max(n, 1))(*([1] * n if algos is None else [int(a) for a in algos]))
        P = ctypes.c_void_p * max(n, 1)
        self._px = P(*[d.data_ptr() for d in self.datas])
        self._pk = P(*[k.data_ptr() for k in self.kernels])
        self._py = P(*[y.data_ptr() for y in self.outs])
        h = ctypes.c_void_p()
        st = L.ndconv_batch_create(probs, n, self.algos, self._px, self._pk, self._py, ctypes.byref(h))
        if st:
            raise RuntimeError(_abi.last_error())
        self._h = h

    def info(self):
        v = (ctypes.c_int64 * 8)()
        _abi.lib().ndconv_batch_info(self._h, v)
        return dict(zip(INFO_FIELDS, list(v)))

    def run(self, graph=True, stream=None):
        s = stream if stream is not None else torch.cuda.current_stream()
        st = _abi.lib().ndconv_batch_run(self._h, 1 if graph else 0, ctypes.c_void_p(s.cuda_stream))
        if st:
            raise RuntimeError(_abi.last_error())
        return self.outs

    def run_plain(self, stream=None):
        s = stream if stream is not None else torch.cuda.current_stream()
        st = _abi.lib().ndconv_batch_run_plain(self._h, ctypes.c_void_p(s.cuda_stream))
        if st:
            raise RuntimeError(_abi.last_error())
        return self.outs

    def check(self, stream=None):
        s = stream if stream is not None else torch.cuda.current_stream()
        st = _abi.lib().ndconv_batch_status(self._h, ctypes.c_void_p(s.cuda_stream))
        if st:
            raise RuntimeError(_abi.last_error())

    def status(self, stream=None):
        """ndconv_batch_status: 0, or the error code (ERR_TIMEOUT when a queue
        wait ran out), without raising."""
        s = stream if stream is not None else torch.cuda.current_stream()
        return _abi.lib().ndconv_batch_status(self._h, ctypes.c_void_p(s.cuda_stream))

    def set_wait_limit(self, polls):
        """Poll bound of the queue's dependency waits (<= 0: the default)."""
        st = _abi.lib().ndconv_batch_set_wait_limit(self._h, int(polls))
        if st:
            raise RuntimeError(_abi.last_error())

    def stall_one_wait(self, enable):
        """Test hook: the first waiting task waits on a counter nothing bumps."""
        st = _abi.lib().ndconv_batch_stall_one_wait(self._h, 1 if enable else 0)
        if st:
            raise RuntimeError(_abi.last_error())

    def close(self):
        if getattr(self, "_h", None):
            _abi.lib().ndconv_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
