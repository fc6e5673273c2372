"""Known-answer channels: geometry with closed-form H, shared by the oracle
test (tests/test_oracle_kat.py) and the GPU test (tests/test_gpu_kat.py).

Free space (max_reflection 0): every verified (Tx, Rx) pair has
    H = bp_rx bp_tx lambda / (4 pi d) exp(-j 2 pi d / lambda),
d the Tx-Rx distance, isotropic patterns (type 0) here
(optixPathTracer.cu:396-416 for the amplitude, :263-264 for the phase).

One mirror (max_reflection 1, a 100 m square reflector with a constant
reflection magnitude r over all angle bins): the one-bounce contribution is
    r lambda / (4 pi d') exp(-j 2 pi d' / lambda),
d' the distance from the Tx image to the Rx (the triangle edges are far
above sqrt(d lambda / 2), so the far-field split of :369-389 never applies).
"""
import numpy as np

LAM = 0.005
REFL = 0.5


def _grid(n, half, z):
    xs = np.linspace(-half, half, n)
    g = np.stack(np.meshgrid(xs, xs, indexing="ij"), -1)
    return np.concatenate([g, np.full((n, n, 1), z)], -1).astype(np.float32)


def mirror_scene():
    """A 100 m x 100 m reflector at z = 0 (two triangles), material 0."""
    a, b = -50.0, 50.0
    tris = np.array([[[a, a, 0], [b, a, 0], [b, b, 0]],
                     [[a, a, 0], [b, b, 0], [a, b, 0]]], np.float32)
    mat = np.zeros(2, np.int32)
    mat_prop = np.full((1, 19), REFL, np.float32)
    return tris, mat, mat_prop


def kat_config(max_reflection):
    tris, mat, mat_prop = mirror_scene()
    # one Tx element: with two elements lambda/2 apart, a ray aimed at one can
    # first pass within the 7 mm capture radius of the other
    # (optixPathTracer.cu:442-444), which the closed form does not model
    src = np.array([[[0.3, -0.2, 2.0]]], np.float32)  # [1, 1, 3]
    dst = _grid(16, 4.0, 1.5)
    params = dict(samples_per_launch=1, launch_x=400, launch_y=400, wave_len=LAM,
                  max_reflection=max_reflection, reserve_size=100, src_bptype=0, dst_bptype=0,
                  dst_gridsize=4, src_r=0.5e-5, dst_r=0.06, src_dir=[0.0, 0.0, -1.0],
                  dst_dir=[0.0, 0.0, 0.0])
    return dict(tris=tris, mat=mat, mat_prop=mat_prop, src=src, dst=dst, params=params)


def free_space_h(src, dst):
    s = src.reshape(-1, 3).astype(np.float64)
    r = dst.reshape(-1, 3).astype(np.float64)
    d = np.linalg.norm(s[:, None, :] - r[None, :, :], axis=-1)
    return LAM / (4 * np.pi * d) * np.exp(-2j * np.pi * d / LAM)


def mirror_h(src, dst):
    s = src.reshape(-1, 3).astype(np.float64).copy()
    s[:, 2] = -s[:, 2]  # image across z = 0
    r = dst.reshape(-1, 3).astype(np.float64)
    d = np.linalg.norm(s[:, None, :] - r[None, :, :], axis=-1)
    return REFL * LAM / (4 * np.pi * d) * np.exp(-2j * np.pi * d / LAM)


def check(H0, H1, src, dst):
    """H0: traced with max_reflection 0, H1 with 1.  Every free-space pair
    must be found (the scene is open and the flood fill reaches every cell);
    the reference's own device programs, run on the CPU, lose 3 of the 256
    one-bounce pairs of this geometry (the backward ray fails verification
    at float precision), so at most 2% may be missing there.  Magnitudes to
    1e-5 relative; phases to 5 mrad (free space) and 20 mrad (one bounce):
    float geometry over ~1e3 wavelengths, about 5 um of path."""
    e0 = free_space_h(src, dst)
    e1 = mirror_h(src, dst)
    assert np.all(np.abs(H0) > 0), "free-space path missing for some pair"
    refl = H1 - H0
    found = np.abs(refl) > 0
    assert found.mean() >= 0.98, f"only {found.mean():.3f} of the one-bounce pairs found"
    for got, want, tol in ((H0, e0, 5e-3), (refl[found], e1[found], 2e-2)):
        assert np.max(np.abs(np.abs(got) / np.abs(want) - 1)) < 1e-5
        assert np.max(np.abs(np.angle(got / want))) < tol
