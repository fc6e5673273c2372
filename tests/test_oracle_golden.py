"""The oracle against golden vectors made by the reference itself.

Channel fixtures come from the reference's device programs run on the CPU
(oracle/ref_harness); objective fixtures from the reference go.Model run on
the CPU (tests/golden/make_golden.py).
"""
import ctypes as C
import os

import numpy as np
import pytest

import cases
import objective_oracle as OO
import oracle
from make_golden import digest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name))


def test_tea_lcg_bit_exact():
    g = load("unit_ref.npz")
    L = oracle.lib()
    tea = np.array([L.orc_tea4(int(s), 0) for s in g["seeds"]], np.uint32)
    assert np.array_equal(tea, g["tea"])
    for s, row in zip(g["seeds"][:32], g["rnd_seq"]):
        st = C.c_uint32(int(s))
        got = np.array([L.orc_rnd(C.byref(st)) for _ in range(16)], np.float32)
        assert np.array_equal(got, row)


def test_rand_dir_matches_reference():
    """Directions agree bit for bit except where libm's cosf/sinf (not
    correctly rounded in about 1% of arguments) and the oracle's correctly
    rounded sin/cos differ by an ulp."""
    g = load("unit_ref.npz")
    L = oracle.lib()
    out = np.zeros((len(g["rand_dir_in"]), 3), np.float32)
    for k, (ix, iy, lx, ly) in enumerate(g["rand_dir_in"]):
        st = C.c_uint32(L.orc_tea4(int(ix * ly + iy), 0))
        L.orc_rnd(C.byref(st))
        o = np.zeros(3, np.float32)
        L.orc_rand_dir(C.byref(st), int(ix), int(iy), int(lx), int(ly), o)
        out[k] = o
    exact = np.all(out == g["rand_dir"], axis=1)
    assert exact.mean() > 0.95
    ulp = np.abs(out.view(np.int32) - g["rand_dir"].view(np.int32))
    assert ulp.max() <= 2


def test_sincos_correctly_rounded():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 100
    L = oracle.lib()
    rng = np.random.Generator(np.random.PCG64(3))
    a = (rng.random(3000) * 6.2831855).astype(np.float32)
    a[:4] = [0.0, np.float32(np.pi / 2), np.float32(np.pi), np.float32(2 * np.pi)]
    out = np.zeros(2, np.float32)
    for x in a:
        L.orc_sincos(float(x), out)
        assert out[0] == np.float32(float(mpmath.sin(mpmath.mpf(float(x)))))
        assert out[1] == np.float32(float(mpmath.cos(mpmath.mpf(float(x)))))


def test_beampattern_matches_reference():
    g = load("unit_ref.npz")
    L = oracle.lib()
    for i in range(len(g["bp_d1"])):
        for t in range(4):
            got = L.orc_beampattern(np.ascontiguousarray(g["bp_d1"][i]),
                                    np.ascontiguousarray(g["bp_d2"][i]), t)
            np.testing.assert_allclose(got, g["bp"][i, t], rtol=2e-6, atol=1e-7)


def test_theta_bins_match_reference():
    g = load("unit_ref.npz")
    L = oracle.lib()
    got = np.array([L.orc_theta_id(float(c)) for c in g["theta_cos"]], np.int32)
    assert np.array_equal(got, g["theta_id"])


def test_theta_bin_edges():
    L = oracle.lib()
    for k in range(19):
        deg = 5.0 * k
        c = np.float32(np.cos(np.radians(deg)))
        assert L.orc_theta_id(float(c)) == k
    assert L.orc_theta_id(float("nan")) == 0
    assert L.orc_theta_id(1.0000001) == 0


@pytest.mark.parametrize("name", cases.CHANNEL_CASES)
def test_channel_matches_reference(name):
    g = load(f"chan_{name}.npz")
    c = cases.channel_case(name)
    assert str(g["input_sha"]) == digest(c["tris"], c["mat"], c["mat_prop"], c["src"], c["dst"])
    H, st, paths = oracle.trace_channel(c["tris"], c["mat"], c["mat_prop"], c["src"], c["dst"],
                                        c["params"], nthreads=2)
    assert [st[k] for k in cases.STAT_KEYS] == list(g["stats"])
    assert np.array_equal(paths, g["paths"])
    # the reference accumulates the phase in FP32; the oracle in FP64
    Hr = g["H"]
    pw = np.abs(H.sum(0)) ** 2
    pr = np.abs(Hr.sum(0)) ** 2
    m = (pw > 0) | (pr > 0)
    assert np.array_equal(pw > 0, pr > 0)
    db = 10 * np.log10(pw[m]) - 10 * np.log10(pr[m])
    assert np.abs(db).max() < 0.1
    assert np.linalg.norm(H - Hr) / np.linalg.norm(Hr) < 2e-3


def test_farfield_case_exercises_the_switch():
    """The far-field FSPL split (optixPathTracer.cu:369-389) changes the loss
    of a path only when a segment outruns 2 maxedge^2 / lambda of the
    triangle before it; the other cases never reach it, this one must."""
    c = cases.channel_case("farfield")
    _, st, _ = oracle.trace_channel(c["tris"], c["mat"], c["mat_prop"], c["src"], c["dst"],
                                    c["params"], nthreads=2)
    assert st["farfield"] > 0.02 * st["rx_paths"]
    t = cases.channel_case("pen_l3")
    _, st0, _ = oracle.trace_channel(t["tris"], t["mat"], t["mat_prop"], t["src"], t["dst"],
                                     t["params"], nthreads=2)
    assert st0["farfield"] == 0


@pytest.mark.parametrize("name", cases.OBJECTIVE_CASES)
def test_objective_matches_reference_model(name):
    g = load(f"obj_{name}.npz")
    c = cases.objective_case(name)
    ch = c["channels"]
    assert str(g["input_sha"]) == digest(*[ch[k] for k in sorted(ch)], c["theta"], *c["phi"])
    A = OO.antenna_amplitude(c["code_num"], c["theta"].shape[1])
    mp = [c["max_phase_deg"] / 180 * np.pi] * c["n_ms"]
    drop = g["drop"]
    if c["n_ms"] <= 1 and c["max_ms_reflex"] <= 1:
        Ha = ch.get("src_to_ms{0}") if c["n_ms"] else None
        Hr = ch.get("ms{0}_to_dst") if c["n_ms"] else None
        phi = c["phi"][0] if c["n_ms"] else None
        loss, gth, gphi, ex = OO.objective(ch["src_to_dst"], Ha, Hr, phi, c["theta"], A, c["w"],
                                           drop, mp[0] if mp else 2 * np.pi)
        np.testing.assert_allclose(ex["amp"], g["recv_amp"], rtol=2e-4, atol=1e-9)
        np.testing.assert_allclose(loss, g["loss"], rtol=1e-5)
        np.testing.assert_allclose(gth, g["grad_theta"], rtol=2e-3,
                                   atol=2e-3 * np.abs(g["grad_theta"]).max())
        if gphi is not None:
            np.testing.assert_allclose(gphi, g["grad_phi0"], rtol=2e-3,
                                       atol=2e-3 * np.abs(g["grad_phi0"]).max())
    else:
        H = OO.composite_channel(ch, c["phi"], mp, c["max_ms_reflex"])
        W = A * np.exp(-1j * c["theta"].astype(np.float64))
        amp = np.abs(W @ H)
        np.testing.assert_allclose(amp, g["recv_amp"], rtol=2e-4, atol=1e-9)
        loss, _ = OO.loss_from_cap(OO.capacity(amp), drop, c["w"])
        np.testing.assert_allclose(loss, g["loss"], rtol=1e-5)


def test_objective_adjoint_finite_differences():
    c = cases.objective_case("c30")
    ch = c["channels"]
    A = OO.antenna_amplitude(c["code_num"], 36)
    drop = np.zeros(c["code_num"], bool)
    drop[[3, 17]] = True
    args = (ch["src_to_dst"], ch["src_to_ms{0}"], ch["ms{0}_to_dst"])
    phi = c["phi"][0].astype(np.float64)
    th = c["theta"].astype(np.float64)
    loss, gth, gphi, _ = OO.objective(*args, phi, th, A, 0.5, drop)
    rng = np.random.Generator(np.random.PCG64(0))
    h = 1e-6
    for m in rng.integers(0, len(phi), 8):
        p1, p2 = phi.copy(), phi.copy()
        p1[m] += h
        p2[m] -= h
        fd = (OO.objective(*args, p1, th, A, 0.5, drop)[0]
              - OO.objective(*args, p2, th, A, 0.5, drop)[0]) / (2 * h)
        assert abs(fd - gphi[m]) <= 1e-4 * max(1.0, abs(gphi[m]))
    for _ in range(8):
        i, j = rng.integers(0, 30), rng.integers(1, 35)
        t1, t2 = th.copy(), th.copy()
        t1[i, j] += h
        t2[i, j] -= h
        fd = (OO.objective(*args, phi, t1, A, 0.5, drop)[0]
              - OO.objective(*args, phi, t2, A, 0.5, drop)[0]) / (2 * h)
        assert abs(fd - gth[i, j]) <= 1e-4 * max(1.0, abs(gth[i, j]))


def test_torch_objective_baseline_matches_oracle():
    """The timed CPU baseline of the objective (the reference's method:
    PyTorch complex64 + autograd) agrees with the FP64 restatement."""
    import torch
    rng = np.random.Generator(np.random.PCG64(5))
    S, M, R, Cn = 8, 64, 200, 4

    def cn(*sh):
        return ((rng.normal(size=sh) + 1j * rng.normal(size=sh)) * 1e-4).astype(np.complex64)
    Hd, Ha, Hr = cn(S, R), cn(S, M), cn(M, R)
    phi = rng.uniform(0, 2 * np.pi, M).astype(np.float32)
    W = (cn(Cn, S) * 1e4).astype(np.complex64)
    lo, gWo, gpo = OO.objective_from_weights(Hd, Ha, Hr, phi, W, 0.5, np.zeros(Cn, bool))
    t = torch.as_tensor
    loss, gW, gp = OO.torch_objective_step(torch, t(Hd), t(Ha), t(Hr), t(phi), t(W), 0.5)
    assert abs(float(loss) - lo) <= 1e-4 * abs(lo)
    assert np.abs(gW.numpy() - gWo).max() <= 1e-3 * np.abs(gWo).max()
    assert np.abs(gp.numpy() - gpo).max() <= 1e-3 * np.abs(gpo).max()
