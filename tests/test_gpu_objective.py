"""CUDA objective + adjoint against the FP64 oracle and against the
reference go.Model (golden fixtures)."""
import os

import numpy as np
import pytest
import torch

import cases
import objective_oracle as OO

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def obj():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from automs_gb300 import objective as O
    return O


def cuda(x):
    return torch.as_tensor(x, device="cuda")


@pytest.mark.parametrize("name", ["c1", "c30", "noms"])
def test_fused_objective_vs_oracle(obj, name):
    c = cases.objective_case(name)
    ch = c["channels"]
    A = OO.antenna_amplitude(c["code_num"], c["theta"].shape[1])
    drop = np.zeros(c["code_num"], bool)
    if c["code_num"] > 2:
        drop[1] = True
    mp = c["max_phase_deg"] / 180 * np.pi
    Ha = ch.get("src_to_ms{0}") if c["n_ms"] else None
    Hr = ch.get("ms{0}_to_dst") if c["n_ms"] else None
    phi = c["phi"][0] if c["n_ms"] else None
    loss_o, gth_o, gphi_o, ex = OO.objective(ch["src_to_dst"], Ha, Hr, phi, c["theta"], A, c["w"],
                                             drop, mp)
    theta = cuda(c["theta"]).requires_grad_(True)
    W = cuda(A.astype(np.float32)) * torch.exp(-1j * theta)
    ph = cuda(phi).requires_grad_(True) if phi is not None else None
    loss, recv = obj.capacity_objective(W, cuda(ch["src_to_dst"]), cuda(Ha) if Ha is not None else None,
                                        cuda(Hr) if Hr is not None else None, ph, mp, c["w"],
                                        cuda(drop), return_recv=True)
    loss.backward()
    np.testing.assert_allclose(float(loss.detach()), loss_o, rtol=1e-4)
    np.testing.assert_allclose(recv.cpu().numpy(), ex["amp"], rtol=1e-4, atol=1e-9)
    g = theta.grad.cpu().numpy()
    np.testing.assert_allclose(g, gth_o, rtol=1e-3, atol=1e-3 * np.abs(gth_o).max())
    if ph is not None:
        gp = ph.grad.cpu().numpy()
        np.testing.assert_allclose(gp, gphi_o, rtol=1e-3, atol=1e-3 * np.abs(gphi_o).max())


@pytest.mark.parametrize("S,M,R,C", [(1, 1, 1, 1), (1, 0, 5, 1), (3, 5, 7, 64), (16, 64, 201, 1),
                                     (4, 9, 33, 2), (2, 17, 4097, 3)])
def test_objective_edge_shapes_vs_oracle(obj, S, M, R, C):
    """Degenerate and ragged shapes through the direct call: one element
    everywhere, no metasurface, the largest codebook (64 codes), an odd Rx
    count (no streaming tiles: the split path), two codes (the streaming
    path's second bucket) and a column count one past a tile, against the
    FP64 oracle."""
    rng = np.random.Generator(np.random.PCG64(1000 + S * 7 + M * 11 + R + C))
    lam = 3e8 / 60e9

    def cn(*sh):
        d = rng.uniform(2.0, 15.0, size=sh)
        g = (rng.normal(size=sh) + 1j * rng.normal(size=sh)) / np.sqrt(2)
        return (g * lam / (4 * np.pi * d)).astype(np.complex64)
    Hd = cn(S, R)
    Ha, Hr = (cn(S, M), cn(M, R)) if M else (None, None)
    phi = rng.uniform(0, 2 * np.pi, M).astype(np.float32) if M else None
    theta = rng.uniform(0, 2 * np.pi, (C, S)).astype(np.float32)
    A = OO.antenna_amplitude(C, S)
    drop = np.zeros(C, bool)
    if C > 2:
        drop[C // 2] = True
    mp, w = 2 * np.pi, 1.0 / R
    loss_o, gth_o, gphi_o, ex = OO.objective(Hd, Ha, Hr, phi, theta, A, w, drop, mp)
    th = cuda(theta).requires_grad_(True)
    W = cuda(A.astype(np.float32)) * torch.exp(-1j * th)
    ph = cuda(phi).requires_grad_(True) if M else None
    loss, recv = obj.capacity_objective(W, cuda(Hd), cuda(Ha) if M else None,
                                        cuda(Hr) if M else None, ph, mp, w, cuda(drop),
                                        return_recv=True)
    loss.backward()
    np.testing.assert_allclose(float(loss.detach()), loss_o, rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(recv.cpu().numpy(), ex["amp"], rtol=1e-4, atol=1e-9)
    # with one AP element |Y| does not depend on theta: the exact gradient is
    # zero and FP32 leaves rounding noise of the loss's scale times 2^-24
    floor = 1e-6 * max(1.0, abs(loss_o))
    g = th.grad.cpu().numpy()
    np.testing.assert_allclose(g, gth_o, rtol=1e-3, atol=1e-3 * np.abs(gth_o).max() + floor)
    if M:
        gp = ph.grad.cpu().numpy()
        np.testing.assert_allclose(gp, gphi_o, rtol=1e-3, atol=1e-3 * np.abs(gphi_o).max() + floor)


@pytest.mark.parametrize("name", cases.OBJECTIVE_CASES)
def test_model_matches_reference_model(obj, name):
    """automs_gb300.objective.Model against go.Model run by the reference
    (same inputs, same dropout rows)."""
    from automs_gb300.geometry import Metasurface
    g = np.load(os.path.join(GOLD, f"obj_{name}.npz"))
    c = cases.objective_case(name)
    chans = {k: cuda(v) for k, v in c["channels"].items()}
    ms = [Metasurface(None, None, None, None, None, c["max_phase_deg"]) for _ in range(c["n_ms"])]
    m = obj.Model(name, chans, ms, max_ms_reflex=c["max_ms_reflex"], code_num=c["code_num"],
                  w=c["w"], drop_rate=0.0)
    with torch.no_grad():
        m.antenna_theta.copy_(cuda(c["theta"]))
        for i in range(c["n_ms"]):
            m.ms_theta[i].copy_(cuda(c["phi"][i]))
    m.drop_rate = 0.0
    W = m.antenna_A * torch.exp(-1j * m.antenna_theta)
    if m._single_hop():
        ch = m.channels[0]
        args = (ch["src_to_ms{0}"], ch["ms{0}_to_dst"], m.ms_theta[0], ms[0].max_phase) \
            if c["n_ms"] else (None, None, None, 2 * np.pi)
        loss = obj.capacity_objective(W, ch["src_to_dst"], args[0], args[1], args[2], args[3],
                                      c["w"], cuda(g["drop"]))
    else:
        # several metasurfaces: Model.forward (library path products and the
        # stacked tensor-core evaluation) with the reference's dropout rows
        m.drop_rate = 0.1
        mask = torch.from_numpy(np.where(g["drop"], 0.0, 0.5).astype(np.float32))
        real_rand = torch.rand
        torch.rand = lambda *a, **k: mask.clone()
        try:
            loss = m.forward()
        finally:
            torch.rand = real_rand
    loss.backward()
    np.testing.assert_allclose(float(loss.detach()), float(g["loss"]), rtol=2e-4)
    gt = g["grad_theta"]
    np.testing.assert_allclose(m.antenna_theta.grad.cpu().numpy(), gt, rtol=5e-3,
                               atol=5e-3 * np.abs(gt).max())
    for i in range(c["n_ms"]):
        gp = g[f"grad_phi{i}"]
        np.testing.assert_allclose(m.ms_theta[i].grad.cpu().numpy(), gp, rtol=5e-3,
                                   atol=5e-3 * np.abs(gp).max())


def test_objective_config_size(obj):
    """The S=16, M=1024, R=4096 plain objective (C=1) against the oracle."""
    rng = np.random.Generator(np.random.PCG64(11))
    S, M, R = 16, 1024, 4096
    Hd = cases._cn(rng, (S, R))
    Ha = cases._cn(rng, (S, M))
    Hr = cases._cn(rng, (M, R))
    phi = rng.uniform(0, 2 * np.pi, M).astype(np.float32)
    wv = (rng.normal(size=S) + 1j * rng.normal(size=S)).astype(np.complex64)
    wv /= np.linalg.norm(wv)
    loss_o, gW_o, gphi_o = OO.mean_capacity(Hd, Ha, Hr, phi, wv)
    w = cuda(wv).requires_grad_(True)
    p = cuda(phi).requires_grad_(True)
    loss = obj.mean_capacity(w, cuda(Hd), cuda(Ha), cuda(Hr), p)
    loss.backward()
    np.testing.assert_allclose(float(loss.detach()), loss_o, rtol=1e-5)
    np.testing.assert_allclose(w.grad.cpu().numpy(), gW_o, rtol=1e-3, atol=1e-3 * np.abs(gW_o).max())
    np.testing.assert_allclose(p.grad.cpu().numpy(), gphi_o, rtol=1e-3,
                               atol=1e-3 * np.abs(gphi_o).max())


def test_optimize_model_decreases_loss(obj):
    from automs_gb300.geometry import Metasurface
    c = cases.objective_case("c30")
    chans = {k: cuda(v) for k, v in c["channels"].items()}
    torch.manual_seed(0)
    m = obj.Model("t", chans, [Metasurface(None, None, None, None, None, 300)], max_ms_reflex=1,
                  code_num=30, w=0.5)
    obj.optimize_model(m, step=30)
    assert m.loss_list[-1] < m.loss_list[0]


def test_coverage_db(obj):
    from automs_gb300 import tracer
    rng = np.random.Generator(np.random.PCG64(5))
    H = (rng.normal(size=(4, 300)) + 1j * rng.normal(size=(4, 300))).astype(np.complex64) * 1e-3
    H[:, 7] = 0
    out = tracer.coverage_db(cuda(H), threshold=-150.0).cpu().numpy()
    with np.errstate(divide="ignore"):  # column 7 is zero: -inf, clamped below
        ref = 20 * np.log10(np.abs(H.sum(0).astype(np.complex128)))
    ref = np.maximum(np.where(np.isnan(ref), -150.0, ref), -150.0)
    np.testing.assert_allclose(out, ref, atol=1e-4)


def _tc_inputs(c, C=None):
    ch = c["channels"]
    Cc = c["code_num"] if C is None else C
    theta = c["theta"][:Cc]
    A = OO.antenna_amplitude(Cc, theta.shape[1])
    drop = np.zeros(Cc, bool)
    if Cc > 2:
        drop[1] = True
    mp = c["max_phase_deg"] / 180 * np.pi
    return ch, theta, A, drop, mp


def _cfg1_codes(C=60, seed=7):
    """S=16 AP, 32x32 metasurface, 64x64 Rx with a C-code codebook."""
    rng = np.random.Generator(np.random.PCG64(seed))
    S, M, R = 16, 1024, 4096
    ch = {"src_to_dst": cases._cn(rng, (S, R)), "src_to_ms{0}": cases._cn(rng, (S, M)),
          "ms{0}_to_dst": cases._cn(rng, (M, R))}
    return dict(channels=ch, theta=rng.uniform(0, 2 * np.pi, size=(C, S)).astype(np.float32),
                phi=[rng.uniform(0, 2 * np.pi, size=M).astype(np.float32)], n_ms=1,
                code_num=C, w=1.0 / R, max_phase_deg=360.0)


@pytest.mark.parametrize("name", ["c1", "c30", "cfg1_c60"])
def test_tensor_core_plan_vs_oracle(obj, name):
    """Tensor-core (3xBF16, FP32 accumulation) evaluation against the FP64
    oracle: loss and |Y| to 1e-4 relative, gradients to 1e-3 of their scale
    (the 3xBF16 products carry about 1e-5 relative error)."""
    c = _cfg1_codes() if name == "cfg1_c60" else cases.objective_case(name)
    ch, theta_np, A, drop, mp = _tc_inputs(c)
    Hd, Ha, Hr = ch["src_to_dst"], ch["src_to_ms{0}"], ch["ms{0}_to_dst"]
    phi = c["phi"][0]
    loss_o, gth_o, gphi_o, ex = OO.objective(Hd, Ha, Hr, phi, theta_np, A, c["w"], drop, mp)
    plan = obj.ObjectivePlan(cuda(Hd), cuda(Ha), cuda(Hr), c_max=64)
    theta = cuda(theta_np).requires_grad_(True)
    W = cuda(A.astype(np.float32)) * torch.exp(-1j * theta)
    ph = cuda(phi).requires_grad_(True)
    loss, recv = obj.capacity_objective(W, cuda(Hd), cuda(Ha), cuda(Hr), ph, mp, c["w"],
                                        cuda(drop), return_recv=True, plan=plan)
    loss.backward()
    np.testing.assert_allclose(float(loss.detach()), loss_o, rtol=1e-4)
    np.testing.assert_allclose(recv.cpu().numpy(), ex["amp"], rtol=1e-4,
                               atol=1e-4 * np.abs(ex["amp"]).max())
    g = theta.grad.cpu().numpy()
    np.testing.assert_allclose(g, gth_o, rtol=1e-3, atol=1e-3 * np.abs(gth_o).max())
    gp = ph.grad.cpu().numpy()
    np.testing.assert_allclose(gp, gphi_o, rtol=1e-3, atol=1e-3 * np.abs(gphi_o).max())
    plan.close()


@pytest.mark.parametrize("name,c_max", [("c1", 1), ("cfg1_c1", 1), ("cfg1_c2", 2)])
def test_streaming_plan_vs_oracle(obj, name, c_max):
    """Plans made with C_max <= 2 stream a transposed FP32 copy of the
    channels (one contiguous block per tile): same tolerances as the direct
    path against the FP64 oracle."""
    if name == "c1":
        c = cases.objective_case("c1")
    else:
        c = _cfg1_codes(C=c_max, seed=9)
    ch, theta_np, A, drop, mp = _tc_inputs(c)
    Hd, Ha, Hr = ch["src_to_dst"], ch["src_to_ms{0}"], ch["ms{0}_to_dst"]
    phi = c["phi"][0]
    loss_o, gth_o, gphi_o, ex = OO.objective(Hd, Ha, Hr, phi, theta_np, A, c["w"], drop, mp)
    plan = obj.ObjectivePlan(cuda(Hd), cuda(Ha), cuda(Hr), c_max=c_max)
    theta = cuda(theta_np).requires_grad_(True)
    W = cuda(A.astype(np.float32)) * torch.exp(-1j * theta)
    ph = cuda(phi).requires_grad_(True)
    for _ in range(2):  # a second call reuses the plan's scratch and counters
        loss, recv = obj.capacity_objective(W, cuda(Hd), cuda(Ha), cuda(Hr), ph, mp, c["w"],
                                            cuda(drop), return_recv=True, plan=plan)
    loss.backward()
    np.testing.assert_allclose(float(loss.detach()), loss_o, rtol=1e-4)
    np.testing.assert_allclose(recv.cpu().numpy(), ex["amp"], rtol=1e-4,
                               atol=1e-4 * np.abs(ex["amp"]).max())
    g = theta.grad.cpu().numpy()
    np.testing.assert_allclose(g, gth_o, rtol=1e-3, atol=1e-3 * np.abs(gth_o).max())
    gp = ph.grad.cpu().numpy()
    np.testing.assert_allclose(gp, gphi_o, rtol=1e-3, atol=1e-3 * np.abs(gphi_o).max())
    plan.close()


def test_tensor_core_plan_matches_cuda_core_path(obj):
    """Same evaluation on the plan and on the FP32 CUDA-core path, the plan
    reused across calls with different C, phi and dropout."""
    c = _cfg1_codes(C=48, seed=11)
    ch = c["channels"]
    Hd, Ha, Hr = (cuda(ch[k]) for k in ("src_to_dst", "src_to_ms{0}", "ms{0}_to_dst"))
    plan = obj.ObjectivePlan(Hd, Ha, Hr, c_max=48)
    assert plan.nbytes > 0
    rng = np.random.Generator(np.random.PCG64(5))
    for C in (48, 5, 1, 33):
        th = cuda(rng.uniform(0, 2 * np.pi, size=(C, 16)).astype(np.float32))
        W = torch.exp(-1j * th)
        phi = cuda(rng.uniform(0, 2 * np.pi, size=1024).astype(np.float32))
        drop = cuda(rng.random(C) < 0.2)
        outs = []
        for p in (plan, None):
            Wg = W.clone().requires_grad_(True)
            pg = phi.clone().requires_grad_(True)
            loss, recv = obj.capacity_objective(Wg, Hd, Ha, Hr, pg, 2 * np.pi, 0.5, drop,
                                                return_recv=True, plan=p)
            loss.backward()
            outs.append((float(loss.detach()), recv, Wg.grad, pg.grad))
        (l1, r1, w1, p1), (l2, r2, w2, p2) = outs
        assert abs(l1 - l2) <= 1e-4 * abs(l2)
        assert torch.allclose(r1, r2, rtol=1e-4, atol=1e-4 * float(r2.abs().max()))
        assert float((w1 - w2).abs().max()) <= 1e-3 * float(w2.abs().max())
        assert float((p1 - p2).abs().max()) <= 1e-3 * float(p2.abs().max())
    plan.close()


def test_plan_with_long_columns_uses_tensor_cores(obj):
    """C_max = 1 with M + S above the streaming kernel's 4096 rows: the plan
    falls back to the tensor-core mode and still matches the oracle."""
    rng = np.random.Generator(np.random.PCG64(21))
    S, M, R = 16, 4096, 256
    ch = {"src_to_dst": cases._cn(rng, (S, R)), "src_to_ms{0}": cases._cn(rng, (S, M)),
          "ms{0}_to_dst": cases._cn(rng, (M, R))}
    c = dict(channels=ch, theta=rng.uniform(0, 2 * np.pi, size=(1, S)).astype(np.float32),
             phi=[rng.uniform(0, 2 * np.pi, size=M).astype(np.float32)], n_ms=1, code_num=1,
             w=1.0 / R, max_phase_deg=360.0)
    ch, theta_np, A, drop, mp = _tc_inputs(c)
    Hd, Ha, Hr = ch["src_to_dst"], ch["src_to_ms{0}"], ch["ms{0}_to_dst"]
    phi = c["phi"][0]
    loss_o, gth_o, gphi_o, ex = OO.objective(Hd, Ha, Hr, phi, theta_np, A, c["w"], drop, mp)
    plan = obj.ObjectivePlan(cuda(Hd), cuda(Ha), cuda(Hr), c_max=1)
    theta = cuda(theta_np).requires_grad_(True)
    W = cuda(A.astype(np.float32)) * torch.exp(-1j * theta)
    ph = cuda(phi).requires_grad_(True)
    loss = obj.capacity_objective(W, cuda(Hd), cuda(Ha), cuda(Hr), ph, mp, c["w"], cuda(drop),
                                  plan=plan)
    loss.backward()
    np.testing.assert_allclose(float(loss.detach()), loss_o, rtol=1e-4)
    gp = ph.grad.cpu().numpy()
    np.testing.assert_allclose(gp, gphi_o, rtol=1e-3, atol=1e-3 * np.abs(gphi_o).max())
    plan.close()


def test_tensor_core_plan_errors(obj):
    from automs_gb300._lib import AmsError
    c = cases.objective_case("c30")
    ch = c["channels"]
    Hd, Ha, Hr = (cuda(ch[k]) for k in ("src_to_dst", "src_to_ms{0}", "ms{0}_to_dst"))
    with pytest.raises(AmsError):
        obj.ObjectivePlan(Hd, Ha, Hr, c_max=65)
    plan = obj.ObjectivePlan(Hd, Ha, Hr, c_max=8)
    W = torch.ones(9, Hd.shape[0], dtype=torch.complex64, device="cuda")
    phi = torch.zeros(Ha.shape[1], device="cuda")
    with pytest.raises(AmsError):
        obj.capacity_objective(W, Hd, Ha, Hr, phi, plan=plan)
    plan.close()


def test_tensor_core_plan_config3_shape_vs_oracle(obj):
    """The 3xBF16 tensor-core plan at the full channel-set shape (S=16,
    M=32x32, R=256x256, a 60-code codebook) against the FP64 oracle: loss
    and |Y| to 1e-4 relative, gradients to 1e-3 of their scale; the measured
    errors are printed."""
    rng = np.random.Generator(np.random.PCG64(31))
    S, M, R, C = 16, 1024, 65536, 60
    ch = {"src_to_dst": cases._cn(rng, (S, R)), "src_to_ms{0}": cases._cn(rng, (S, M)),
          "ms{0}_to_dst": cases._cn(rng, (M, R))}
    c = dict(channels=ch, theta=rng.uniform(0, 2 * np.pi, size=(C, S)).astype(np.float32),
             phi=[rng.uniform(0, 2 * np.pi, size=M).astype(np.float32)], n_ms=1, code_num=C,
             w=1.0 / R, max_phase_deg=360.0)
    ch, theta_np, A, drop, mp = _tc_inputs(c)
    Hd, Ha, Hr = ch["src_to_dst"], ch["src_to_ms{0}"], ch["ms{0}_to_dst"]
    phi = c["phi"][0]
    loss_o, gth_o, gphi_o, ex = OO.objective(Hd, Ha, Hr, phi, theta_np, A, c["w"], drop, mp)
    dHd, dHa, dHr = cuda(Hd), cuda(Ha), cuda(Hr)
    plan = obj.ObjectivePlan(dHd, dHa, dHr, c_max=C)
    theta = cuda(theta_np).requires_grad_(True)
    W = cuda(A.astype(np.float32)) * torch.exp(-1j * theta)
    ph = cuda(phi).requires_grad_(True)
    loss, recv = obj.capacity_objective(W, dHd, dHa, dHr, ph, mp, c["w"], cuda(drop),
                                        return_recv=True, plan=plan)
    loss.backward()
    obj.check_status(plan)
    amp = recv.cpu().numpy()
    g, gp = theta.grad.cpu().numpy(), ph.grad.cpu().numpy()
    e_loss = abs(float(loss.detach()) - loss_o) / abs(loss_o)
    e_amp = np.abs(amp - ex["amp"]).max() / np.abs(ex["amp"]).max()
    e_th = np.abs(g - gth_o).max() / np.abs(gth_o).max()
    e_ph = np.abs(gp - gphi_o).max() / np.abs(gphi_o).max()
    print(f"3xBF16 at R=65536 C=60 vs FP64: loss {e_loss:.2e}, |Y| {e_amp:.2e}, "
          f"dtheta {e_th:.2e}, dphi {e_ph:.2e}")
    assert e_loss < 1e-4 and e_amp < 1e-4
    assert e_th < 1e-3 and e_ph < 1e-3
    plan.close()


@pytest.mark.parametrize("path", ["direct", "stream_plan", "tensor_core_plan"])
def test_wait_timeout_is_reported(obj, path):
    """A bounded wait that runs out (injected on the host: the kernels wait
    exactly as usual) makes the call's loss and gradients NaN and the status
    call report it; the next call is clean and matches an undisturbed one."""
    from automs_gb300._lib import AmsError, lib
    rng = np.random.Generator(np.random.PCG64(41))
    S, M, R = 16, 1024, 4096
    C = 60 if path == "tensor_core_plan" else 1
    Hd, Ha, Hr = (cuda(cases._cn(rng, sh)) for sh in ((S, R), (S, M), (M, R)))
    W = torch.exp(-1j * cuda(rng.uniform(0, 2 * np.pi, size=(C, S)).astype(np.float32)))
    phi = cuda(rng.uniform(0, 2 * np.pi, size=M).astype(np.float32))
    plan = None if path == "direct" else obj.ObjectivePlan(Hd, Ha, Hr, c_max=C)

    def run():
        Wg = W.clone().requires_grad_(True)
        pg = phi.clone().requires_grad_(True)
        loss = obj.capacity_objective(Wg, Hd, Ha, Hr, pg, 2 * np.pi, 1.0 / R, plan=plan)
        loss.backward()
        return float(loss.detach()), Wg.grad.clone(), pg.grad.clone()
    clean = run()
    obj.check_status(plan)
    lib().ams_debug_inject_wait_timeout(1)
    bad = run()
    assert np.isnan(bad[0])
    assert torch.isnan(bad[1]).all() and torch.isnan(bad[2]).all()
    with pytest.raises(AmsError) as ei:
        obj.check_status(plan)
    assert ei.value.status == 7
    again = run()
    obj.check_status(plan)
    assert again[0] == clean[0]
    assert torch.equal(again[1], clean[1]) and torch.equal(again[2], clean[2])
    if plan is not None:
        plan.close()


@pytest.mark.parametrize("name", cases.OBJECTIVE_CASES)
def test_postprocess_matches_reference_model(obj, name, monkeypatch):
    """Model.postprocess (go.py:89-97) against go.Model's: code phases rounded
    to pi/2 steps, metasurface phases reduced modulo max_phase, then the
    forward pass: Model.result (|Y|), Model.max_code_ids and the loss, with
    the reference's dropout draw replayed."""
    from automs_gb300.geometry import Metasurface
    g = np.load(os.path.join(GOLD, f"post_{name}.npz"))
    c = cases.objective_case(name)
    chans = {k: cuda(v) for k, v in c["channels"].items()}
    ms = [Metasurface(None, None, None, None, None, c["max_phase_deg"]) for _ in range(c["n_ms"])]
    m = obj.Model(name, chans, ms, max_ms_reflex=c["max_ms_reflex"], code_num=c["code_num"],
                  w=c["w"], drop_rate=0.0)
    with torch.no_grad():
        m.antenna_theta.copy_(cuda(c["theta"]))
        for i in range(c["n_ms"]):
            m.ms_theta[i].copy_(cuda(g[f"phi_in{i}"]))
    m.drop_rate = 0.1
    drawn = torch.from_numpy(g["rand"])
    monkeypatch.setattr(torch, "rand", lambda *a, **k: drawn.clone())
    m.postprocess()
    monkeypatch.undo()
    np.testing.assert_array_equal(m.antenna_theta.detach().cpu().numpy(), g["theta_post"])
    for i in range(c["n_ms"]):
        np.testing.assert_allclose(m.ms_theta[i].detach().cpu().numpy(), g[f"phi_post{i}"],
                                   rtol=0, atol=2e-6)
        assert float(m.ms_theta[i].detach().max()) < ms[i].max_phase
    res = m.result.cpu().numpy()
    np.testing.assert_allclose(res, g["result"], rtol=1e-4, atol=1e-4 * np.abs(g["result"]).max())
    # the strongest code per Rx, wherever it leads the runner-up clearly
    top2 = np.sort(g["result"], axis=0)[-2:] if g["result"].shape[0] > 1 else None
    ids = m.max_code_ids.cpu().numpy()
    clear = (np.ones(ids.shape, bool) if top2 is None
             else (top2[1] - top2[0]) > 1e-3 * np.abs(g["result"]).max())
    assert clear.mean() > 0.9
    np.testing.assert_array_equal(ids[clear], g["max_code_ids"][clear])
    np.testing.assert_allclose(float(m.loss.detach()), float(g["loss"]), rtol=2e-4)


def _reference_multihop_loss(torch_, ch, W, phis, max_phases, reflex, w, drop):
    """go.py:107-157 get_channel + go.py:159-226 forward (capacity mode) in
    float64 / complex128 on the CPU with autograd: the reference's method."""
    import itertools
    n = len(phis)
    H = ch["src_to_dst"]
    for L in range(1, reflex + 1):
        for path in itertools.product(range(n), repeat=L):
            if any(path[i] == path[i + 1] for i in range(L - 1)):
                continue
            msc = ch["src_to_ms{%d}" % path[0]]
            for i, m in enumerate(path):
                msc = msc * torch_.exp(1j * torch_.remainder(phis[m], max_phases[m]))
                if i == L - 1:
                    msc = msc @ ch["ms{%d}_to_dst" % m]
                else:
                    nx = path[i + 1]
                    msc = msc @ (ch["ms{%d}_to_ms{%d}" % (m, nx)] if m < nx
                                 else ch["ms{%d}_to_ms{%d}" % (nx, m)].T)
            H = H + msc
    Y = W @ H
    cap = torch_.log2(1.0 + (Y.abs() + OO.EPS32) ** 2 / OO.N0)
    cap = cap * (~drop)[:, None]
    mx, _ = cap.max(0)
    masked = cap * (cap != mx[None, :])
    return -w * mx.sum() + torch_.linalg.norm(masked)


def test_multihop_objective_vs_reference_autograd(obj):
    """Three metasurfaces, paths of up to three hops (transposed hops
    included): loss and gradients of Model.forward (library path products +
    stacked tensor-core evaluation) against the reference's method in
    float64 with autograd."""
    from automs_gb300.geometry import Metasurface
    rng = np.random.Generator(np.random.PCG64(77))
    S, R, C, Ms = 8, 300, 6, [40, 24, 32]
    ch = {"src_to_dst": cases._cn(rng, (S, R))}
    for i, M in enumerate(Ms):
        ch["src_to_ms{%d}" % i] = cases._cn(rng, (S, M)) * 30
        ch["ms{%d}_to_dst" % i] = cases._cn(rng, (M, R)) * 30
    for i in range(3):
        for j in range(i + 1, 3):
            ch["ms{%d}_to_ms{%d}" % (i, j)] = cases._cn(rng, (Ms[i], Ms[j])) * 30
    theta = rng.uniform(0, 2 * np.pi, size=(C, S)).astype(np.float32)
    phis = [rng.uniform(0, 4 * np.pi, size=M).astype(np.float32) for M in Ms]
    max_deg = [360.0, 300.0, 270.0]
    drop = np.zeros(C, bool)
    drop[2] = True
    ms = [Metasurface(None, None, None, None, None, d) for d in max_deg]
    m = obj.Model("t", {k: cuda(v) for k, v in ch.items()}, ms, max_ms_reflex=3, code_num=C,
                  w=0.7, drop_rate=0.1)
    with torch.no_grad():
        m.antenna_theta.copy_(cuda(theta))
        for i in range(3):
            m.ms_theta[i].copy_(cuda(phis[i]))
    for p in m.parameters():
        p.grad = None
    mask = torch.from_numpy(np.where(drop, 0.0, 0.5).astype(np.float32))
    real_rand = torch.rand
    torch.rand = lambda *a, **k: mask.clone()
    try:
        loss = m.forward()
    finally:
        torch.rand = real_rand
    loss.backward()
    obj.check_status()
    # reference: float64 autograd on the CPU
    t64 = {k: torch.from_numpy(v.astype(np.complex128)) for k, v in ch.items()}
    th = torch.from_numpy(theta.astype(np.float64)).requires_grad_(True)
    ph = [torch.from_numpy(p.astype(np.float64)).requires_grad_(True) for p in phis]
    A = torch.from_numpy(OO.antenna_amplitude(C, S))
    W64 = A * torch.exp(-1j * th)
    ref = _reference_multihop_loss(torch, t64, W64, ph, [d / 180 * np.pi for d in max_deg], 3,
                                   0.7, torch.from_numpy(drop))
    ref.backward()
    np.testing.assert_allclose(float(loss.detach()), float(ref.detach()), rtol=1e-4)
    gt = th.grad.numpy()
    np.testing.assert_allclose(m.antenna_theta.grad.cpu().numpy(), gt, rtol=1e-3,
                               atol=1e-3 * np.abs(gt).max())
    for i in range(3):
        gp = ph[i].grad.numpy()
        np.testing.assert_allclose(m.ms_theta[i].grad.cpu().numpy(), gp, rtol=1e-3,
                                   atol=1e-3 * np.abs(gp).max())


def test_cgemm_ops(obj):
    """ams_cgemm against numpy for each operand mode, with accumulation."""
    rng = np.random.Generator(np.random.PCG64(5))
    mk = lambda *sh: (rng.normal(size=sh) + 1j * rng.normal(size=sh)).astype(np.complex64)
    f = {0: lambda x: x, 1: lambda x: x.T, 2: lambda x: x.conj().T, 3: lambda x: x.conj()}
    for opA in range(4):
        for opB in range(4):
            A = mk(37, 50) if opA in (0, 3) else mk(50, 37)
            B = mk(50, 29) if opB in (0, 3) else mk(29, 50)
            C0 = mk(37, 29)
            out = cuda(C0)
            obj.cgemm(cuda(A), cuda(B), opA, opB, out=out, accumulate=True)
            ref = C0.astype(np.complex128) + f[opA](A).astype(np.complex128) @ f[opB](B)
            np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())
