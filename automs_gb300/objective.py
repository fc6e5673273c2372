"""Phase-map objective: fused CUDA forward + adjoint behind autograd, and a
Model / optimize_model pair with the interface of go.py:27-336.

The objective and its hand-written adjoint run in libams.so
(ams_objective_fwd_bwd); this module only wires them into
torch.autograd.Function so that Adam (as in optimize_model, go.py:296-336)
drives them.
"""
import ctypes as C
import itertools
import math
import random

import torch
import torch.nn as nn

from ._lib import call, lib


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _c64(t):
    t = t.to(torch.complex64)
    return t if t.is_contiguous() else t.contiguous()


class ObjectivePlan:
    """Tensor-core objective for a fixed channel set (ams_objective_plan_*).

    [H_r; H_d] are converted once into BF16 hi/lo pairs; each evaluation then
    runs the forward and adjoint contractions as tcgen05 GEMMs (3xBF16
    products, FP32 accumulation, relative error about 1e-5).  For codebooks
    (C up to c_max <= 64) evaluated many times, as in optimize_model."""

    def __init__(self, H_d, H_a, H_r, c_max=64):
        lib()
        self.Hd, self.Ha, self.Hr = _c64(H_d.detach()), _c64(H_a.detach()), _c64(H_r.detach())
        self.S, self.R = self.Hd.shape
        self.M = self.Ha.shape[1]
        if self.Ha.shape[0] != self.S or tuple(self.Hr.shape) != (self.M, self.R):
            raise ValueError("channel shapes do not match: H_d [S,R], H_a [S,M], H_r [M,R]")
        self.c_max = int(c_max)
        h = C.c_void_p()
        call("ams_objective_plan_create", _ptr(self.Hd), _ptr(self.Ha), _ptr(self.Hr), self.S,
             self.M, self.R, self.c_max, _stream(), C.byref(h))
        self._h = h

    @property
    def nbytes(self):
        return int(lib().ams_objective_plan_bytes(self._h)) if self._h else 0

    def close(self):
        if getattr(self, "_h", None):
            lib().ams_objective_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CapacityObjective(torch.autograd.Function):
    """loss(W, phi) of go.py:159-226 for one metasurface hop (or none):
    Y = W H_d + ((W H_a) o e^{j (phi mod max_phase)}) H_r.
    The adjoint is computed in the same call; backward only scales it."""

    @staticmethod
    def forward(ctx, W, phi, H_d, H_a, H_r, max_phase, w, drop, want_recv, plan=None):
        Cc, S = W.shape
        R = H_d.shape[1]
        ms = H_a is not None
        M = H_a.shape[1] if ms else 0
        Wc = _c64(W.detach())
        Hd = _c64(H_d.detach())
        Ha = _c64(H_a.detach()) if ms else None
        Hr = _c64(H_r.detach()) if ms else None
        ph = phi.detach().to(torch.float32).contiguous() if ms else None
        loss = torch.empty((), dtype=torch.float32, device=W.device)
        gW = torch.empty_like(Wc)
        gphi = torch.empty(M, dtype=torch.float32, device=W.device) if ms else None
        need_gy = H_d.requires_grad
        gY = torch.empty(Cc, R, dtype=torch.complex64, device=W.device) if need_gy else None
        recv = torch.empty(Cc, R, dtype=torch.float32, device=W.device) if want_recv else None
        dr = drop.to(device=W.device, dtype=torch.uint8).contiguous() if drop is not None else None
        if plan is not None:
            if not ms or (plan.S, plan.M, plan.R) != (S, M, R):
                raise ValueError("the plan was made for other channel shapes")
            call("ams_objective_plan_fwd_bwd", plan._h, _ptr(ph), float(max_phase), _ptr(Wc), Cc,
                 float(w), _ptr(dr), _ptr(loss), _ptr(gW), _ptr(gphi), _ptr(gY), _ptr(recv),
                 _stream())
        else:
            call("ams_objective_fwd_bwd", _ptr(Hd), _ptr(Ha), _ptr(Hr), _ptr(ph),
                 float(max_phase), _ptr(Wc), S, M, R, Cc, float(w), _ptr(dr), _ptr(loss),
                 _ptr(gW), _ptr(gphi), _ptr(gY), _ptr(recv), _stream())
        ctx.save_for_backward(gW, gphi if gphi is not None else torch.empty(0, device=W.device),
                              gY if gY is not None else torch.empty(0, device=W.device), Wc)
        ctx.ms = ms
        ctx.need_gy = need_gy
        ctx.w_dtype = W.dtype
        if recv is not None:
            ctx.mark_non_differentiable(recv)
            return loss, recv
        return loss, torch.empty(0, device=W.device)

    @staticmethod
    def backward(ctx, gl, _grecv):
        gW, gphi, gY, Wc = ctx.saved_tensors
        dW = (gW * gl).to(ctx.w_dtype) if ctx.needs_input_grad[0] else None
        dphi = gphi * gl if (ctx.ms and ctx.needs_input_grad[1]) else None
        dHd = None
        if ctx.need_gy and ctx.needs_input_grad[2]:
            # Y = W H_d  =>  dL/dH_d = W^H dL/dY (torch's complex convention)
            dHd = (Wc.conj().transpose(0, 1) @ gY) * gl
        return dW, dphi, dHd, None, None, None, None, None, None, None


def capacity_objective(W, H_d, H_a=None, H_r=None, phi=None, max_phase=2 * math.pi, w=1.0,
                       drop=None, return_recv=False, plan=None):
    """Differentiable objective.  W [C,S] complex, H_d [S,R], H_a [S,M],
    H_r [M,R] complex64 CUDA tensors, phi [M] float, drop [C] bool.  With an
    ObjectivePlan made from these channels the tensor-core path runs."""
    lib()
    loss, recv = CapacityObjective.apply(W, phi, H_d, H_a, H_r, max_phase, w, drop, return_recv,
                                         plan)
    return (loss, recv) if return_recv else loss


def cgemm(A, B, opA=0, opB=0, out=None, accumulate=False):
    """op(A) op(B) (+ out) on the library's complex GEMM (ams_cgemm): 2-D
    complex64 CUDA tensors; op 0 as is, 1 transposed, 2 conjugate
    transposed, 3 conjugated."""
    A, B = _c64(A), _c64(B)
    m, k = (A.shape[0], A.shape[1]) if opA in (0, 3) else (A.shape[1], A.shape[0])
    kb, n = (B.shape[0], B.shape[1]) if opB in (0, 3) else (B.shape[1], B.shape[0])
    if k != kb:
        raise ValueError(f"inner dimensions differ: {k} vs {kb}")
    if out is None:
        out = (torch.zeros if accumulate else torch.empty)(m, n, dtype=torch.complex64,
                                                         device=A.device)
    call("ams_cgemm", m, n, k, _ptr(A), A.shape[1], opA, _ptr(B), B.shape[1], opB, _ptr(out),
         out.shape[1], int(accumulate), _stream())
    return out


class StackedPlan:
    """Tensor-core objective plan over several metasurfaces'
    channels (ams_objective_plan_create_stacked): the MS->Rx rows of every
    metasurface stacked in one [M, R] block beside H_d."""

    def __init__(self, H_d, H_rs, c_max):
        lib()
        self.Hd = _c64(H_d.detach())
        self.Hr = torch.cat([_c64(h.detach()) for h in H_rs], 0).contiguous()
        self.sizes = [h.shape[0] for h in H_rs]
        self.S, self.R = self.Hd.shape
        self.M = self.Hr.shape[0]
        self.c_max = int(c_max)
        h = C.c_void_p()
        call("ams_objective_plan_create_stacked", _ptr(self.Hd), _ptr(self.Hr), self.S, self.M,
             self.R, self.c_max, _stream(), C.byref(h))
        self._h = h

    close = ObjectivePlan.close
    __del__ = ObjectivePlan.__del__


def ms_paths(n_ms, max_ms_reflex):
    """Metasurface sequences of get_channel (go.py:112-156): lengths 1 ..
    max_ms_reflex, no metasurface twice in a row."""
    out = []
    for L in range(1, max_ms_reflex + 1):
        for path in itertools.product(range(n_ms), repeat=L):
            if all(path[i] != path[i + 1] for i in range(L - 1)):
                out.append(path)
    return out


class MultiHopObjective(torch.autograd.Function):
    """loss(W, phi) of go.py:107-245 for several metasurfaces and paths up to
    max_ms_reflex hops on the library's kernels: each path's product
    (W H_a^(p0) o e^(p0)) H^(p0 p1) o e^(p1) ... (ams_cgemm) adds to the
    coefficient of its last metasurface's rows, one stacked tensor-core
    evaluation (ams_objective_plan_coef_fwd_bwd) gives the loss and dL/dU,
    and the backward pass chains dL/dU through the products (ams_cgemm)."""

    @staticmethod
    def forward(ctx, W, phi_cat, plan, chans, max_phases, paths, w, drop, want_recv):
        Wc = _c64(W.detach())
        Cc = Wc.shape[0]
        off = [0]
        for m in plan.sizes:
            off.append(off[-1] + m)
        e = []
        for i, mp in enumerate(max_phases):
            ph = torch.remainder(phi_cat.detach()[off[i]:off[i + 1]].to(torch.float32), mp)
            e.append(torch.polar(torch.ones_like(ph), ph).to(torch.complex64))
        U = torch.zeros(Cc, plan.M, dtype=torch.complex64, device=W.device)
        saved = []
        for path in paths:
            X = cgemm(Wc, chans["src_to_ms{%d}" % path[0]])
            V = X * e[path[0]][None, :]
            nodes = [(path[0], V, None, 0)]
            for prev, m in zip(path[:-1], path[1:]):
                if prev < m:
                    B, op = chans["ms{%d}_to_ms{%d}" % (prev, m)], 0
                else:
                    B, op = chans["ms{%d}_to_ms{%d}" % (m, prev)], 1
                X = cgemm(V, B, opB=op)
                V = X * e[m][None, :]
                nodes.append((m, V, B, op))
            last = path[-1]
            U[:, off[last]:off[last + 1]] += V
            saved.append((path, nodes))
        loss = torch.empty((), dtype=torch.float32, device=W.device)
        gU = torch.empty_like(U)
        gW = torch.empty_like(Wc)
        recv = torch.empty(Cc, plan.R, dtype=torch.float32, device=W.device) if want_recv else None
        dr = drop.to(device=W.device, dtype=torch.uint8).contiguous() if drop is not None else None
        call("ams_objective_plan_coef_fwd_bwd", plan._h, _ptr(U), _ptr(Wc), Cc, float(w), _ptr(dr),
             _ptr(loss), _ptr(gU), _ptr(gW), _ptr(recv), _stream())
        ctx.saved = (saved, e, off, chans)
        ctx.save_for_backward(gU, gW)
        ctx.w_dtype = W.dtype
        if recv is not None:
            ctx.mark_non_differentiable(recv)
            return loss, recv
        return loss, torch.empty(0, device=W.device)

    @staticmethod
    def backward(ctx, gl, _grecv):
        gU, gW = ctx.saved_tensors
        saved, e, off, chans = ctx.saved
        dW = gW * gl
        dphi = torch.zeros(off[-1], dtype=torch.float32, device=gU.device)
        for path, nodes in saved:
            last = path[-1]
            dV = gU[:, off[last]:off[last + 1]] * gl
            for k in range(len(nodes) - 1, -1, -1):
                m, V, B, op = nodes[k]
                dphi[off[m]:off[m + 1]] -= torch.imag(torch.conj(dV) * V).sum(0)
                dX = dV * torch.conj(e[m])[None, :]
                if k > 0:
                    # X = V_prev B (op 0) or V_prev B^T (op 1)
                    dV = cgemm(dX, B, opB=2 if op == 0 else 3)
                else:
                    dW = dW + cgemm(dX, chans["src_to_ms{%d}" % m], opB=2)
        return (dW.to(ctx.w_dtype), dphi, None, None, None, None, None, None, None)


def check_status(plan=None):
    """Raise AmsError if a bounded wait of the last objective call ran out
    (its outputs are then NaN): the last call on `plan`, or with plan=None the
    last direct call on the current device.  Synchronises the stream."""
    h = plan._h if plan is not None else None
    call("ams_objective_status", h if h is not None else C.c_void_p(0), _stream())


def mean_capacity(wvec, H_d, H_a=None, H_r=None, phi=None):
    """-mean over Rx of log2(1 + |y|^2 / N0) with one complex weight vector:
    the reference loss with C = 1, w = 1/R and no dropout."""
    R = H_d.shape[1]
    return capacity_objective(wvec.reshape(1, -1), H_d, H_a, H_r, phi, 2 * math.pi, 1.0 / R)


class Model(nn.Module):
    """go.py:27-245 with the objective on libams.so.

    Same constructor, parameters (antenna_theta [C,S], ms_theta list),
    attributes (loss_list, result, cap, max_code_ids) and loss.  The 10% code
    dropout is drawn with torch.rand on the CPU generator as the reference
    does (go.py:219-220); pass drop_rate=0 to disable it."""

    def __init__(self, name, channels, ms_list, max_ms_reflex=2, code_num=60, w=1.0,
                 global_random=False, drop_rate=0.1, device="cuda", plans=True):
        super().__init__()
        # one metasurface hop: an ObjectivePlan per channel set (made on first
        # use; C <= 2 streams a transposed copy, larger codebooks run on the
        # tensor cores)
        self.use_plans = bool(plans) and code_num <= 64
        self._plans = {}
        if isinstance(channels, dict):
            channels = [channels]
        self.name = name
        self.ms_list = ms_list
        self.max_ms_reflex = max_ms_reflex
        self.channels = [{k: _c64(v.to(device)) for k, v in ch.items()} for ch in channels]
        self.loss_list = []
        self.w = w
        self.global_random = global_random
        self.drop_rate = drop_rate
        S = self.channels[0]["src_to_dst"].shape[0]
        A = torch.ones(code_num, S, dtype=torch.float32, device=device) / math.sqrt(S / 36)
        if S == 36:
            A[:, [0, 5, 30, 35]] = 0
        self.antenna_A = A
        self.antenna_theta = nn.Parameter(
            torch.rand(code_num, S, dtype=torch.float32, device=device) * 2 * torch.pi)
        self.ms_A = []
        self.ms_theta = nn.ParameterList()
        for i in range(len(ms_list)):
            M = self.channels[0]["src_to_ms{%d}" % i].shape[1]
            self.ms_A.append(torch.ones(M, dtype=torch.float32, device=device))
            self.ms_theta.append(torch.zeros(M, dtype=torch.float32, device=device))
        self.forward()

    def postprocess(self):
        """go.py:89-97: theta to pi/2 steps, phi into [0, max_phase)."""
        self.antenna_theta = nn.Parameter(
            torch.round(self.antenna_theta / (torch.pi / 2)) * (torch.pi / 2))
        for i in range(len(self.ms_list)):
            self.ms_theta[i] = self.ms_theta[i] % self.ms_list[i].max_phase
        self.forward()

    def check_status(self):
        """Raise if a bounded wait of the last evaluation ran out."""
        for plan in self._plans.values():
            check_status(plan)
        check_status()

    def pick_channel(self, choose_new=False):
        if self.global_random:
            if choose_new:
                self.picked_channel = random.choice(self.channels)
            return self.picked_channel
        return random.choice(self.channels)

    def _single_hop(self):
        n = len(self.ms_list)
        return n == 0 or self.max_ms_reflex == 0 or (n == 1 and self.max_ms_reflex >= 1)

    def get_channel(self):
        """Composite channel H [S, R] (go.py:107-157), the path products on
        the library's complex GEMM (not differentiable: forward() forms the
        loss and its gradient without it)."""
        channel = self.pick_channel(True)["src_to_dst"]
        for L in range(1, self.max_ms_reflex + 1):
            for path in itertools.product(range(len(self.ms_list)), repeat=L):
                if any(path[i] == path[i + 1] for i in range(L - 1)):
                    continue
                msc = self.pick_channel()["src_to_ms{%d}" % path[0]]
                for i, m in enumerate(path):
                    real = self.ms_theta[m].detach() % self.ms_list[m].max_phase
                    msc = msc * (self.ms_A[m] * torch.exp(1j * real))
                    if i == L - 1:
                        msc = cgemm(msc, self.pick_channel()["ms{%d}_to_dst" % m])
                    else:
                        nx = path[i + 1]
                        if m < nx:
                            msc = cgemm(msc, self.pick_channel()["ms{%d}_to_ms{%d}" % (m, nx)])
                        else:
                            msc = cgemm(msc, self.pick_channel()["ms{%d}_to_ms{%d}" % (nx, m)],
                                        opB=1)
                channel = channel + msc
        return channel

    def forward(self):
        W = self.antenna_A * torch.exp(-1j * self.antenna_theta)
        C_ = W.shape[0]
        drop = torch.rand(C_) < self.drop_rate if self.drop_rate > 0 else None
        if self._single_hop():
            ch = self.pick_channel(True)
            use_ms = len(self.ms_list) == 1 and self.max_ms_reflex >= 1
            if use_ms:
                plan = None
                if self.use_plans:
                    plan = self._plans.get(id(ch))
                    if plan is None:
                        plan = ObjectivePlan(ch["src_to_dst"], ch["src_to_ms{0}"],
                                             ch["ms{0}_to_dst"], c_max=C_)
                        self._plans[id(ch)] = plan
                loss, recv = capacity_objective(
                    W, ch["src_to_dst"], ch["src_to_ms{0}"], ch["ms{0}_to_dst"], self.ms_theta[0],
                    self.ms_list[0].max_phase, self.w, drop, return_recv=True, plan=plan)
            else:
                loss, recv = capacity_objective(W, ch["src_to_dst"], w=self.w, drop=drop,
                                                return_recv=True)
        else:
            # several metasurfaces / hops: path products on the library's
            # complex GEMM, one stacked tensor-core evaluation
            ch = self.pick_channel(True)
            n = len(self.ms_list)
            plan = self._plans.get(("stacked", id(ch)))
            if plan is None:
                plan = StackedPlan(ch["src_to_dst"], [ch["ms{%d}_to_dst" % i] for i in range(n)],
                                   c_max=C_)
                self._plans[("stacked", id(ch))] = plan
            loss, recv = MultiHopObjective.apply(
                W, torch.cat(list(self.ms_theta)), plan, ch,
                [m.max_phase for m in self.ms_list], ms_paths(n, self.max_ms_reflex), self.w,
                drop, True)
        self.result = recv.detach().clone()
        self.max_code_ids = recv.max(0)[1].detach().clone()
        eps = torch.finfo(torch.float32).eps
        self.cap = torch.log2(1 + (recv + eps) ** 2 / 10 ** (-9)).detach()
        self.loss = loss
        return loss


def optimize_model(model: Model, lr: float = 0.3, step: int = 200, progress=False):
    """go.py:296-336: Adam over the model parameters, best-loss snapshot."""
    opt = torch.optim.Adam(model.parameters(), lr=lr)
    best = float("inf")
    best_theta = None
    best_ms = None
    it = range(step)
    if progress:
        from tqdm import tqdm
        it = tqdm(it)
    for _ in it:
        loss = model()
        lv = loss.item()
        if lv < best:
            best = lv
            best_theta = model.antenna_theta.detach().clone()
            best_ms = [t.detach().clone() for t in model.ms_theta]
        loss.backward()
        opt.step()
        opt.zero_grad()
        model.loss_list.append(lv)
    with torch.no_grad():
        model.antenna_theta.copy_(best_theta)
        for t, b in zip(model.ms_theta, best_ms):
            t.copy_(b)
    model.forward()
    model.check_status()
