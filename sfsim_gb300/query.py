"""Queries of a built atmosphere on the GPU (the C ABI's context functions).

`Context(cfg)` builds the four tables on the current CUDA device and keeps
them there with the point-scatter table summed over the iterations.  Its
methods take and return torch CUDA tensors of shape [n, 3]:
  table(kind, a, b, light)  the lookups sfsim's shaders perform
                            (resources/shaders/atmosphere/*.glsl)
  direct(x, v, l)           rendered in-scatter S + M phase by direct quadrature
`ConditionedSurrogate` is one surrogate network for a family of atmospheres.
"""
from __future__ import annotations

import ctypes

from . import _lib
from .config import AtmoConfig

TRANSMITTANCE_TRACK = 0
TRANSMITTANCE_OUTER = 1
RAY_SCATTER_TRACK = 2
RAY_SCATTER_OUTER = 3
IN_SCATTER = 4


class Context:
    def __init__(self, cfg: AtmoConfig):
        self.cfg = cfg.copy()
        self._L = _lib.load()
        self._ptr = ctypes.c_void_p()
        _lib.check(self._L.sfsim_atmo_context_create(ctypes.byref(self.cfg), ctypes.byref(self._ptr)),
                   "sfsim_atmo_context_create")

    def close(self):
        if self._ptr:
            self._L.sfsim_atmo_context_destroy(self._ptr)
            self._ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def tables(self):
        """Copies of the four tables (.scatter layout) as torch CUDA tensors."""
        import torch
        from .atmosphere_lut import table_shapes
        ptrs = [ctypes.c_void_p() for _ in range(4)]
        _lib.check(self._L.sfsim_atmo_context_tables(self._ptr, *[ctypes.byref(p) for p in ptrs]), "tables")
        out = []
        for p, shape in zip(ptrs, table_shapes(self.cfg)):
            t = torch.empty(shape, dtype=torch.float32, device="cuda")
            n = t.numel() * 4
            torch.cuda.synchronize()
            _cuda_copy(t.data_ptr(), p.value, n)
            out.append(t)
        return out

    def point_scatter_sum(self):
        """The point-scatter table summed over the iterations, [n0,n1,n2,n3,4] (RGB + pad), or None."""
        import torch
        p = ctypes.c_void_p()
        _lib.check(self._L.sfsim_atmo_context_point_scatter_sum(self._ptr, ctypes.byref(p)), "point_scatter_sum")
        if not p.value:
            return None
        s = tuple(self.cfg.ray_scatter_shape) + (4,)
        t = torch.empty(s, dtype=torch.float32, device="cuda")
        _cuda_copy(t.data_ptr(), p.value, t.numel() * 4)
        return t

    def table(self, kind: int, a, b, light=None, weight_bits: int = 0, out=None):
        import torch
        a = a.contiguous().float()
        b = b.contiguous().float()
        light = light.contiguous().float() if light is not None else None
        n = a.shape[0]
        out = out if out is not None else torch.empty((n, 3), dtype=torch.float32, device="cuda")
        st = torch.cuda.current_stream().cuda_stream
        _lib.check(self._L.sfsim_atmo_query_table(self._ptr, kind, n, a.data_ptr(), b.data_ptr(),
                                                  light.data_ptr() if light is not None else None,
                                                  out.data_ptr(), weight_bits, st), "query_table")
        return out

    def attenuation(self, kind: int, light, p, d=None, s=None, incoming=None, amplification: float = 1.0,
                    weight_bits: int = 0, out=None):
        """Attenuation along view rays as the shaders compute it
        (sfsim_atmo_query_attenuation): kind 0 attenuation_outer(light, p, d,
        s[:, 0], incoming rgb), 1 attenuation_track(light, p, d, s, incoming),
        2 attenuation_point(p, incoming) with the eye d, 3
        transmittance_point(p); CUDA tensors in, an [n, 4] RGBA tensor out."""
        import torch
        f = lambda t: t.contiguous().float() if t is not None else None  # noqa: E731
        light, p, d, s, incoming = f(light), f(p), f(d), f(s), f(incoming)
        n = p.shape[0]
        out = out if out is not None else torch.empty((n, 4), dtype=torch.float32, device="cuda")
        ptr = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
        st = torch.cuda.current_stream().cuda_stream
        _lib.check(self._L.sfsim_atmo_query_attenuation(self._ptr, kind, n, ptr(light), ptr(p), ptr(d), ptr(s),
                                                        ptr(incoming), amplification, out.data_ptr(), weight_bits,
                                                        st), "query_attenuation")
        return out

    # -- surrogate -------------------------------------------------------------
    def train_surrogate(self, steps=2000, batch=65536, direct_samples=1 << 20, node_fraction=0.0, lr=1e-3,
                        seed=1, huber_delta=0.0):
        """Trains the surrogate MLP on the GPU against `direct_samples` random
        queries integrated by direct quadrature (node_fraction of each batch
        drawn from the table nodes with a zero correction instead); returns
        the per-step mean squared errors of the log-space correction (numpy)."""
        import numpy as np
        c = _lib.SurrogateConfig(steps, batch, direct_samples, node_fraction, lr, seed, huber_delta)
        hist = np.zeros(max(steps, 1), np.float32)
        _lib.check(self._L.sfsim_atmo_surrogate_train(self._ptr, ctypes.byref(c), hist.ctypes.data), "train")
        return hist[:steps]

    def surrogate_parameters(self, set_to=None):
        import numpy as np
        n = ctypes.c_longlong()
        _lib.check(self._L.sfsim_atmo_surrogate_parameters(self._ptr, None, None, ctypes.byref(n)), "parameters")
        out = np.zeros(n.value, np.float32)
        src = None
        if set_to is not None:
            src = np.ascontiguousarray(set_to, dtype=np.float32)
            assert src.size == n.value
        _lib.check(self._L.sfsim_atmo_surrogate_parameters(self._ptr, out.ctypes.data,
                                                           src.ctypes.data if src is not None else None,
                                                           ctypes.byref(n)), "parameters")
        return out

    def surrogate_gradients(self, coords, targets):
        """Loss and parameter gradients of one batch (numpy in, numpy out)."""
        import numpy as np
        coords = np.ascontiguousarray(coords, dtype=np.float32)
        targets = np.ascontiguousarray(targets, dtype=np.float32)
        n = coords.shape[0]
        grads = np.zeros(self.surrogate_parameters().size, np.float32)
        loss = np.zeros(1, np.float32)
        _lib.check(self._L.sfsim_atmo_surrogate_gradients(self._ptr, n, coords.ctypes.data, targets.ctypes.data,
                                                          loss.ctypes.data, grads.ctypes.data), "gradients")
        return float(loss[0]), grads

    def surrogate(self, x, v, l, threshold=0.0, out=None):
        """Rendered in-scatter from the surrogate-corrected table lookup; with
        threshold > 0 the points whose predicted relative error exceeds it are
        recomputed by direct quadrature.  Returns (out, number recomputed)."""
        import torch
        x = x.contiguous().double()
        v = v.contiguous().double()
        l = l.contiguous().double()
        n = x.shape[0]
        out = out if out is not None else torch.empty((n, 3), dtype=torch.float32, device="cuda")
        nf = ctypes.c_longlong()
        st = torch.cuda.current_stream().cuda_stream
        _lib.check(self._L.sfsim_atmo_query_surrogate(self._ptr, n, x.data_ptr(), v.data_ptr(), l.data_ptr(),
                                                      out.data_ptr(), threshold, ctypes.byref(nf), st), "surrogate")
        return out, nf.value

    def coords(self, x, v, l):
        """The surrogate's coordinates [n, 10] in [0, 1] of the queries: the table coordinates (height,
        elevation, sun elevation, heading), the unclamped sun elevation, the table half and the four
        cell phases of the lookup."""
        import torch
        x = x.contiguous().double()
        v = v.contiguous().double()
        l = l.contiguous().double()
        out = torch.empty((x.shape[0], 10), dtype=torch.float32, device="cuda")
        _lib.check(self._L.sfsim_atmo_query_coords(self._ptr, x.shape[0], x.data_ptr(), v.data_ptr(), l.data_ptr(),
                                                   out.data_ptr(), torch.cuda.current_stream().cuda_stream),
                   "query_coords")
        return out

    def direct(self, x, v, l, out=None):
        import torch
        x = x.contiguous().double()
        v = v.contiguous().double()
        l = l.contiguous().double()
        n = x.shape[0]
        out = out if out is not None else torch.empty((n, 3), dtype=torch.float32, device="cuda")
        st = torch.cuda.current_stream().cuda_stream
        _lib.check(self._L.sfsim_atmo_query_direct(self._ptr, n, x.data_ptr(), v.data_ptr(), l.data_ptr(),
                                                   out.data_ptr(), st), "query_direct")
        return out


def condition_inputs(cfg: AtmoConfig):
    """The conditioned surrogate's eight inputs of an atmosphere (numpy float32)."""
    import numpy as np
    L = _lib.load()
    out = np.zeros(8, np.float32)
    _lib.check(L.sfsim_atmo_condition_inputs(ctypes.byref(cfg), out.ctypes.data), "condition_inputs")
    return out


class ConditionedSurrogate:
    """One surrogate network for a family of atmospheres: the eight inputs of
    `condition_inputs` join the first layer.  `train(contexts, ...)` trains it on
    several built atmospheres; `query(ctx, x, v, l)` corrects any context's
    table lookup (torch CUDA tensors in and out, as Context.surrogate)."""

    def __init__(self, seed: int = 1):
        self._L = _lib.load()
        self._ptr = ctypes.c_void_p()
        _lib.check(self._L.sfsim_atmo_cond_surrogate_create(seed, ctypes.byref(self._ptr)), "cond_surrogate_create")

    def close(self):
        if self._ptr:
            self._L.sfsim_atmo_cond_surrogate_destroy(self._ptr)
            self._ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def train(self, contexts, steps=2000, batch=65536, direct_samples=1 << 18, node_fraction=0.0, lr=1e-3, seed=1,
              huber_delta=0.0):
        """Trains on the contexts (a list of Context sharing one ray-scatter
        shape; direct_samples per context); returns the per-step losses."""
        import numpy as np
        c = _lib.SurrogateConfig(steps, batch, direct_samples, node_fraction, lr, seed, huber_delta)
        arr = (ctypes.c_void_p * len(contexts))(*[ctx._ptr.value for ctx in contexts])
        hist = np.zeros(max(steps, 1), np.float32)
        _lib.check(self._L.sfsim_atmo_cond_surrogate_train(self._ptr, arr, len(contexts), ctypes.byref(c),
                                                           hist.ctypes.data), "cond_surrogate_train")
        return hist[:steps]

    def parameters(self, set_to=None):
        import numpy as np
        n = ctypes.c_longlong()
        _lib.check(self._L.sfsim_atmo_cond_surrogate_parameters(self._ptr, None, None, ctypes.byref(n)), "parameters")
        out = np.zeros(n.value, np.float32)
        src = None
        if set_to is not None:
            src = np.ascontiguousarray(set_to, dtype=np.float32)
            assert src.size == n.value
        _lib.check(self._L.sfsim_atmo_cond_surrogate_parameters(self._ptr, out.ctypes.data,
                                                                src.ctypes.data if src is not None else None,
                                                                ctypes.byref(n)), "parameters")
        return out

    def gradients(self, coords, groups, inputs, targets):
        """Loss and parameter gradients of one batch (numpy in, numpy out)."""
        import numpy as np
        coords = np.ascontiguousarray(coords, dtype=np.float32)
        groups = np.ascontiguousarray(groups, dtype=np.int32)
        inputs = np.ascontiguousarray(inputs, dtype=np.float32)
        targets = np.ascontiguousarray(targets, dtype=np.float32)
        grads = np.zeros(self.parameters().size, np.float32)
        loss = np.zeros(1, np.float32)
        _lib.check(self._L.sfsim_atmo_cond_surrogate_gradients(self._ptr, coords.shape[0], coords.ctypes.data,
                                                               groups.ctypes.data, inputs.shape[0], inputs.ctypes.data,
                                                               targets.ctypes.data, loss.ctypes.data,
                                                               grads.ctypes.data), "cond_gradients")
        return float(loss[0]), grads

    def query(self, ctx, x, v, l, threshold=0.0, out=None):
        """Rendered in-scatter of ctx's atmosphere from its table lookup
        corrected by the network; returns (out, number recomputed)."""
        import torch
        x = x.contiguous().double()
        v = v.contiguous().double()
        l = l.contiguous().double()
        n = x.shape[0]
        out = out if out is not None else torch.empty((n, 3), dtype=torch.float32, device="cuda")
        nf = ctypes.c_longlong()
        st = torch.cuda.current_stream().cuda_stream
        _lib.check(self._L.sfsim_atmo_query_cond_surrogate(self._ptr, ctx._ptr, n, x.data_ptr(), v.data_ptr(),
                                                           l.data_ptr(), out.data_ptr(), threshold, ctypes.byref(nf),
                                                           st), "query_cond_surrogate")
        return out, nf.value


def _cuda_copy(dst: int, src: int, nbytes: int) -> None:
    """Device-to-device copy through torch (no extra CUDA bindings needed)."""
    import torch
    s = torch.cuda.current_stream()
    # wrap the raw pointer as a tensor view through the CUDA array interface
    class _Arr:
        def __init__(self, ptr, n):
            self.__cuda_array_interface__ = {"shape": (n,), "typestr": "|u1", "data": (ptr, False), "version": 3}
    src_t = torch.as_tensor(_Arr(src, nbytes), device="cuda")
    dst_t = torch.as_tensor(_Arr(dst, nbytes), device="cuda")
    dst_t.copy_(src_t)
    s.synchronize()
