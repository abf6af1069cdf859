"""The learned part (include/dem_learned.h): per-pair feature-contact counts
predicted by a 16-64-64-4 MLP trained on the GPU by the library's own BF16 /
FP32 kernels, used to size the polyhedron feature records and to order the
candidate pairs into warp bins.  The exact enumeration still decides every
interaction.

Device buffers are torch CUDA tensors (plain device memory); the arithmetic is
the library's."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A

NIN, NHID, NOUT = 16, 64, 4
NPARAM = NHID * NIN + NHID + NHID * NHID + NHID + NOUT * NHID + NOUT


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


class Learned:
    """MLP operations on the context of a System (polyhedra)."""

    def __init__(self, system):
        self.s = system

    def _chk(self, rc, where):
        self.s._check(rc, where)

    def harvest(self, capacity: int):
        """Inputs (n x 16 float32) and exact labels (n x 4 uint8) of the candidate
        pairs of the current neighbour list, as CUDA tensors."""
        import torch

        x = torch.empty((max(capacity, 1), NIN), dtype=torch.float32, device="cuda")
        y = torch.empty((max(capacity, 1), NOUT), dtype=torch.uint8, device="cuda")
        n, avail = C.c_uint64(), C.c_uint64()
        self._chk(self.s.b.mlp_harvest(self.s.h, _ptr(x), _ptr(y), capacity, C.byref(n), C.byref(avail)),
                  "mlp_harvest")
        return x[: n.value], y[: n.value], int(avail.value)

    def init(self, seed: int = 4, label_means=None) -> None:
        lm = None if label_means is None else (C.c_float * NOUT)(*map(float, label_means))
        self._chk(self.s.b.mlp_init(self.s.h, seed, lm), "mlp_init")

    def params(self) -> np.ndarray:
        p = np.zeros(NPARAM, dtype=np.float32)
        self._chk(self.s.b.mlp_get_params(self.s.h, p.ctypes.data_as(C.POINTER(C.c_float))), "mlp_get_params")
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._chk(self.s.b.mlp_set_params(self.s.h, p.ctypes.data_as(C.POINTER(C.c_float))), "mlp_set_params")

    def rates(self, x):
        import torch

        r = torch.empty((x.shape[0], NOUT), dtype=torch.float32, device="cuda")
        self._chk(self.s.b.mlp_forward(self.s.h, _ptr(x), x.shape[0], _ptr(r)), "mlp_forward")
        return r

    def loss_grad(self, x, y):
        g = np.zeros(NPARAM, dtype=np.float32)
        loss = C.c_double()
        self._chk(self.s.b.mlp_loss_grad(self.s.h, _ptr(x), _ptr(y), x.shape[0],
                                         g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)), "mlp_loss_grad")
        return float(loss.value), g

    def train(self, x, y, epochs: int = 10, batch: int = 65536, lr: float = 1e-3, seed: int = 4) -> list:
        losses = (C.c_double * epochs)()
        self._chk(self.s.b.mlp_train(self.s.h, _ptr(x), _ptr(y), x.shape[0], epochs, batch, lr, seed, losses),
                  "mlp_train")
        return list(losses)

    def stats(self) -> dict:
        u, o, r = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._chk(self.s.b.learned_stats(self.s.h, C.byref(u), C.byref(o), C.byref(r)), "learned_stats")
        return {"units": int(u.value), "overflow": int(o.value), "record_entries": int(r.value)}
