"""Surrogate MLP on libams.so: BF16 tensor-core training and inference.

The network maps a placement descriptor (metasurface position, orientation,
size and a scene occupancy code) to a coarse coverage-gain map; annealing
uses it to rank candidates so that the ray tracer only judges the best.
"""
import ctypes as C

import numpy as np
import torch

from ._lib import call, lib


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def gemm_bf16(A, B, bias=None, relu=False, out16=False):
    """C = A @ B.T on the tensor cores; A [M,K], B [N,K] bf16 CUDA tensors."""
    A = A.contiguous()
    B = B.contiguous()
    M, K = A.shape
    N = B.shape[0]
    C32 = torch.empty(M, N, dtype=torch.float32, device=A.device)
    C16 = torch.empty(M, N, dtype=torch.bfloat16, device=A.device) if out16 else None
    call("ams_gemm_bf16", _ptr(A), _ptr(B), M, N, K, _ptr(bias), int(relu), _ptr(C32), _ptr(C16),
         _stream())
    return (C32, C16) if out16 else C32


class MLP:
    """dims = [d_in, hidden..., d_out]; widths after the input are multiples of 128."""

    def __init__(self, dims, max_batch=4096, seed=0):
        lib()
        self.dims = list(dims)
        self.max_batch = max_batch
        arr = (C.c_int * len(dims))(*dims)
        self._h = C.c_void_p()
        call("ams_mlp_create", arr, len(dims), int(max_batch), C.c_ulonglong(seed), _stream(),
             C.byref(self._h))
        n = C.c_longlong()
        call("ams_mlp_params", self._h, C.c_void_p(0), 0, C.byref(n), _stream())
        self.n_params = n.value

    def close(self):
        if self._h:
            lib().ams_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, X, T=None):
        X = X.to(device="cuda", dtype=torch.float32).contiguous()
        if X.shape[1] != self.dims[0] or X.shape[0] > self.max_batch:
            raise ValueError("bad input shape")
        if T is not None:
            T = T.to(device="cuda", dtype=torch.float32).contiguous()
            if T.shape != (X.shape[0], self.dims[-1]):
                raise ValueError("bad target shape")
        return X, T

    def forward(self, X):
        outs = []
        for i in range(0, X.shape[0], self.max_batch):
            Xi, _ = self._chk(X[i:i + self.max_batch])
            Y = torch.empty(Xi.shape[0], self.dims[-1], device="cuda")
            call("ams_mlp_forward", self._h, _ptr(Xi), Xi.shape[0], _ptr(Y), _stream())
            outs.append(Y)
        return torch.cat(outs, 0)

    __call__ = forward

    def train_step(self, X, T, lr=1e-3):
        X, T = self._chk(X, T)
        loss = torch.empty((), device="cuda")
        call("ams_mlp_train_step", self._h, _ptr(X), _ptr(T), X.shape[0], float(lr), _ptr(loss),
             _stream())
        return loss

    def gradients(self, X, T):
        X, T = self._chk(X, T)
        loss = torch.empty((), device="cuda")
        g = torch.empty(self.n_params, device="cuda")
        call("ams_mlp_gradients", self._h, _ptr(X), _ptr(T), X.shape[0], _ptr(loss), _ptr(g),
             _stream())
        return loss, g

    def get_params(self):
        p = torch.empty(self.n_params, device="cuda")
        call("ams_mlp_params", self._h, _ptr(p), 0, None, _stream())
        return p

    def set_params(self, p):
        p = p.to(device="cuda", dtype=torch.float32).contiguous()
        if p.numel() != self.n_params:
            raise ValueError("parameter count mismatch")
        call("ams_mlp_params", self._h, _ptr(p), 1, None, _stream())

    def state_dict(self):
        """Everything needed to resume training: widths, FP32 parameters,
        Adam moments and step (CPU tensors)."""
        m1 = torch.empty(self.n_params, device="cuda")
        m2 = torch.empty(self.n_params, device="cuda")
        step = C.c_longlong(0)
        call("ams_mlp_adam_state", self._h, _ptr(m1), _ptr(m2), C.byref(step), 0, _stream())
        return {"dims": list(self.dims), "params": self.get_params().cpu(), "adam_m": m1.cpu(),
                "adam_v": m2.cpu(), "adam_step": int(step.value)}

    def load_state_dict(self, sd):
        if list(sd["dims"]) != self.dims:
            raise ValueError(f"checkpoint widths {sd['dims']} != {self.dims}")
        self.set_params(sd["params"])
        m1 = sd["adam_m"].to(device="cuda", dtype=torch.float32).contiguous()
        m2 = sd["adam_v"].to(device="cuda", dtype=torch.float32).contiguous()
        if m1.numel() != self.n_params or m2.numel() != self.n_params:
            raise ValueError("Adam state size mismatch")
        step = C.c_longlong(int(sd["adam_step"]))
        call("ams_mlp_adam_state", self._h, _ptr(m1), _ptr(m2), C.byref(step), 1, _stream())

    def save(self, path):
        torch.save(self.state_dict(), path)

    @classmethod
    def load(cls, path, max_batch=4096):
        sd = torch.load(path, map_location="cpu")
        net = cls(sd["dims"], max_batch=max_batch)
        net.load_state_dict(sd)
        return net

    def fit(self, X, T, epochs=10, batch=1024, lr=1e-3, seed=0, lr_decay=1.0):
        """Minibatch Adam over (X, T); returns the per-epoch mean losses."""
        g = torch.Generator(device="cpu").manual_seed(seed)
        n = X.shape[0]
        hist = []
        for ep in range(epochs):
            perm = torch.randperm(n, generator=g)
            tot, cnt = 0.0, 0
            for i in range(0, n, batch):
                idx = perm[i:i + batch].to(X.device)
                loss = self.train_step(X[idx], T[idx], lr)
                tot += float(loss) * idx.numel()
                cnt += idx.numel()
            hist.append(tot / cnt)
            lr *= lr_decay
        return hist
