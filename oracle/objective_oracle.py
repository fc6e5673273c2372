"""FP64 restatement of the phase-map objective and its adjoint.

TEST INFRASTRUCTURE ONLY: the checker for the CUDA objective kernels.

Follows go.py:107-157 (Model.get_channel) and go.py:159-245 (Model.forward,
loss_mode "capacity"), channels in the reference orientation:
  H_d = src_to_dst [S,R], H_a = src_to_ms{i} [S,M], H_r = ms{i}_to_dst [M,R].
Code weights W = A * exp(-j theta) [C,S]  (go.py:60-75, 163).
The random 10% code dropout (go.py:219-220) is an explicit boolean row mask.

Complex gradients use torch's convention dL/dRe + j dL/dIm.
"""
import itertools

import numpy as np

N0 = 10.0 ** (-90 / 10)                 # noise floor -90 dBm in mW, go.py:183-184
EPS32 = float(np.finfo(np.float32).eps)  # go.py:181
LN2 = np.log(2.0)


def antenna_amplitude(code_num, antenna_num):
    """A = 1/sqrt(S/36), the four corners of a 6x6 AP zeroed (go.py:60-66)."""
    A = np.full((code_num, antenna_num), 1.0 / np.sqrt(antenna_num / 36.0))
    if antenna_num == 36:
        A[:, [0, 5, 30, 35]] = 0.0
    return A


def ms_phase(phi, max_phase_rad):
    """phi mod max_phase with Python/torch remainder semantics (go.py:133)."""
    return np.mod(np.asarray(phi, np.float64), max_phase_rad)


def composite_channel(channels, phis, max_phases, max_ms_reflex):
    """H = H_d + sum over MS paths of the path products (go.py:107-157)."""
    H = channels["src_to_dst"].astype(np.complex128)
    n_ms = len(phis)
    for L in range(1, max_ms_reflex + 1):
        for path in itertools.product(range(n_ms), repeat=L):
            if any(path[i] == path[i + 1] for i in range(L - 1)):
                continue
            acc = channels["src_to_ms{%d}" % path[0]].astype(np.complex128)
            for i, m in enumerate(path):
                acc = acc * np.exp(1j * ms_phase(phis[m], max_phases[m]))[None, :]
                if i == L - 1:
                    acc = acc @ channels["ms{%d}_to_dst" % m].astype(np.complex128)
                else:
                    nxt = path[i + 1]
                    if m < nxt:
                        acc = acc @ channels["ms{%d}_to_ms{%d}" % (m, nxt)].astype(np.complex128)
                    else:
                        acc = acc @ channels["ms{%d}_to_ms{%d}" % (nxt, m)].astype(np.complex128).T
            H = H + acc
    return H


def capacity(amp):
    """log2(1 + (|y| + eps)^2 / N0), go.py:181-188."""
    return np.log2(1.0 + (amp + EPS32) ** 2 / N0)


def loss_from_cap(cap, drop, w):
    """loss = -w * sum_r max_c cap' + ||cap' * mask||_F, go.py:219-226.
    Returns (loss, dL/dcap)."""
    rc = cap.copy()
    rc[drop] = 0.0
    idx = np.argmax(rc, axis=0)
    mx = rc[idx, np.arange(rc.shape[1])]
    mask = rc != mx[None, :]
    masked = rc * mask
    nrm = np.sqrt(np.sum(masked ** 2))
    loss = -w * mx.sum() + nrm
    g = np.zeros_like(rc)
    g[idx, np.arange(rc.shape[1])] += -w
    if nrm > 0:
        g += mask * masked / nrm
    g[drop] = 0.0
    return loss, g


def objective(H_d, H_a, H_r, phi, theta, A, w, drop, max_phase=2 * np.pi):
    """Single-metasurface objective and adjoint (max_ms_reflex = 1).

    H_a/H_r may be None for the no-metasurface case.  Returns
    (loss, dL/dtheta [C,S], dL/dphi [M] or None, extras dict)."""
    H_d = np.asarray(H_d, np.complex128)
    W = np.asarray(A, np.float64) * np.exp(-1j * np.asarray(theta, np.float64))
    Y = W @ H_d
    if H_a is not None:
        H_a = np.asarray(H_a, np.complex128)
        H_r = np.asarray(H_r, np.complex128)
        e = np.exp(1j * ms_phase(phi, max_phase))
        V = W @ H_a
        U = V * e[None, :]
        Y = Y + U @ H_r
    amp = np.abs(Y)
    cap = capacity(amp)
    loss, g_cap = loss_from_cap(cap, np.asarray(drop, bool), w)
    a = amp + EPS32
    g_amp = g_cap * (2.0 * a / N0) / ((1.0 + a * a / N0) * LN2)
    with np.errstate(invalid="ignore", divide="ignore"):
        G_Y = np.where(amp > 0, g_amp * Y / amp, 0.0)
    G_W = G_Y @ H_d.conj().T
    g_phi = None
    if H_a is not None:
        G_U = G_Y @ H_r.conj().T
        g_phi = -np.imag(np.conj(G_U) * U).sum(axis=0)
        G_V = G_U * np.conj(e)[None, :]
        G_W = G_W + G_V @ H_a.conj().T
    g_theta = np.imag(np.conj(G_W) * W)
    return loss, g_theta, g_phi, dict(Y=Y, amp=amp, cap=cap, G_W=G_W, W=W)


def objective_from_weights(H_d, H_a, H_r, phi, W, w, drop, max_phase=2 * np.pi):
    """Same objective with complex code weights W [C,S] given directly.
    Returns (loss, dL/dW (dRe + j dIm), dL/dphi)."""
    W = np.asarray(W, np.complex128)
    A = np.abs(W)
    theta = -np.angle(W)
    loss, _, g_phi, ex = objective(H_d, H_a, H_r, phi, theta, A, w, drop, max_phase)
    return loss, ex["G_W"], g_phi


def mean_capacity(H_d, H_a, H_r, phi, wvec):
    """Plain objective -mean_R log2(1 + |y|^2/N0) with one complex weight
    vector (C = 1, no dropout): the reference loss with w = 1/R."""
    R = H_d.shape[1]
    loss, gW, gphi = objective_from_weights(H_d, H_a, H_r, phi, np.asarray(wvec)[None, :],
                                            1.0 / R, np.zeros(1, bool))
    return loss, gW[0], gphi


def torch_objective_step(torch, H_d, H_a, H_r, phi, W, w, max_phase=2 * np.pi):
    """One forward + backward of the reference's own method: PyTorch complex64
    tensors and autograd (go.py:107-157 get_channel with one metasurface hop,
    go.py:159-245 forward in "capacity" mode, no dropout), on whatever device
    the tensors live.  Used as the timed CPU baseline of the objective.
    Returns (loss, dL/dW, dL/dphi)."""
    W = W.detach().clone().requires_grad_(True)
    phi = phi.detach().clone().requires_grad_(True)
    p = torch.remainder(phi, max_phase)
    H = H_d + (H_a * torch.exp(1j * p.to(H_a.dtype))[None, :]) @ H_r
    Y = W @ H
    cap = torch.log2(1.0 + (Y.abs() + EPS32) ** 2 / N0)
    mx, _ = cap.max(0)
    masked = cap * (cap != mx[None, :])
    loss = -w * mx.sum() + torch.linalg.norm(masked)
    loss.backward()
    return loss.detach(), W.grad, phi.grad
