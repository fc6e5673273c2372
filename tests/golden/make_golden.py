"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run where the reference tree is mounted, naming it in AMS_REFERENCE_ROOT:

    AMS_REFERENCE_ROOT=<reference tree> python tests/golden/make_golden.py

Three sources:
  * channel fixtures: the reference's own device programs
    (optixPathTracer.cu) compiled for the CPU by oracle/ref_harness and run
    on seeded synthetic scenes (cases in tests/golden/cases.py);
  * objective fixtures: the reference's own go.Model (go.py:27-245) imported
    with stub matplotlib / numpy-stl modules and run on the CPU, loss and
    autograd gradients recorded;
  * geometry fixtures: the reference's geometry helpers (go.py:248-512,
    1309-1338) on seeded inputs, imported the same way.
Outputs are small .npz files; the inputs are regenerated from the case
definitions, whose sha256 is stored alongside to catch generator drift.
"""
import contextlib
import ctypes as C
import hashlib
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)
REF = os.environ.get("AMS_REFERENCE_ROOT")

import cases  # noqa: E402
import oracle  # noqa: E402


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def make_channel_fixtures(names=cases.CHANNEL_CASES):
    for name in names:
        c = cases.channel_case(name)
        H, st, paths = oracle.ref_trace_channel(c["tris"], c["mat"], c["mat_prop"],
                                                c["src"], c["dst"], c["params"])
        np.savez_compressed(
            os.path.join(HERE, f"chan_{name}.npz"),
            H=H, paths=paths,
            stats=np.array([st[k] for k in cases.STAT_KEYS], np.int64),
            input_sha=np.array(digest(c["tris"], c["mat"], c["mat_prop"], c["src"], c["dst"])))
        print(name, st)


def make_unit_fixtures():
    R = oracle.ref_lib()
    rng = np.random.Generator(np.random.PCG64(7))
    seeds = rng.integers(0, 2**32, size=256, dtype=np.uint64).astype(np.uint32)
    tea = np.array([R.ref_tea4(int(s), 0) for s in seeds], np.uint32)
    rnd_seq = []
    for s in seeds[:32]:
        st = C.c_uint32(int(s))
        rnd_seq.append([R.ref_rnd(C.byref(st)) for _ in range(16)])
    rnd_seq = np.array(rnd_seq, np.float32)
    dirs = []
    rd_in = []
    for k in range(512):
        lx, ly = int(rng.integers(1, 1200)), int(rng.integers(1, 1200))
        ix, iy = int(rng.integers(0, lx)), int(rng.integers(0, ly))
        st = C.c_uint32(R.ref_tea4(ix * ly + iy, 0))
        R.ref_rnd(C.byref(st))  # the src draw precedes the direction
        out = np.zeros(3, np.float32)
        R.ref_rand_dir(C.byref(st), ix, iy, lx, ly, out)
        dirs.append(out)
        rd_in.append([ix, iy, lx, ly])
    d1 = rng.normal(size=(400, 3)).astype(np.float32)
    d2 = rng.normal(size=(400, 3)).astype(np.float32)
    bp = np.zeros((400, 4), np.float32)
    for i in range(400):
        for t in range(4):
            bp[i, t] = R.ref_beampattern(np.ascontiguousarray(d1[i]), np.ascontiguousarray(d2[i]), t)
    n = rng.normal(size=(200, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    n = n.astype(np.float32)
    a = rng.uniform(-5, 5, size=(200, 3)).astype(np.float32)
    m0 = rng.uniform(-2, 2, size=(200, 12)).astype(np.float32)
    m1 = m0.copy()
    for i in range(200):
        row = np.ascontiguousarray(m1[i])
        R.ref_image_update(row, np.ascontiguousarray(n[i]), np.ascontiguousarray(a[i]))
        m1[i] = row
    cosv = rng.uniform(-1, 1, size=4000).astype(np.float32)
    tid = np.array([R.ref_theta_id(float(c)) for c in cosv], np.int32)
    np.savez_compressed(os.path.join(HERE, "unit_ref.npz"), seeds=seeds, tea=tea,
                        rnd_seq=rnd_seq, rand_dir=np.array(dirs, np.float32),
                        rand_dir_in=np.array(rd_in, np.int64), bp_d1=d1, bp_d2=d2, bp=bp,
                        img_n=n, img_a=a, img_m0=m0, img_m1=m1, theta_cos=cosv, theta_id=tid)
    print("unit fixtures written")


class StubMesh:
    """Stand-in for numpy-stl's mesh.Mesh (go.py:9, 700): from_file reads a
    binary STL record by record with struct (independent of the package's
    numpy reader, scenes.read_stl) and exposes .vectors [n, 3, 3] float32."""

    def __init__(self, vectors):
        self.vectors = vectors

    @classmethod
    def from_file(cls, path):
        import struct
        with open(path, "rb") as f:
            data = f.read()
        (n,) = struct.unpack_from("<I", data, 80)
        out = np.zeros((n, 3, 3), np.float32)
        for i in range(n):
            rec = struct.unpack_from("<12fH", data, 84 + 50 * i)
            out[i] = np.asarray(rec[3:12], np.float32).reshape(3, 3)
        return cls(out)


# ------------------------------------------------------------ objective
@contextlib.contextmanager
def reference_go_on_cpu():
    """Import the reference go.py with stub plotting / STL modules and with
    its hard-coded device="cuda" redirected to the CPU."""
    import torch
    stubs = {}
    for name in ("matplotlib", "matplotlib.pyplot", "stl", "stl.mesh"):
        stubs[name] = types.ModuleType(name)
    stubs["stl"].mesh = stubs["stl.mesh"]
    stubs["stl.mesh"].Mesh = StubMesh
    stubs["matplotlib"].pyplot = stubs["matplotlib.pyplot"]
    saved_mods = {k: sys.modules.get(k) for k in stubs}
    sys.modules.update(stubs)
    factories = ("ones", "zeros", "rand", "tensor", "linspace")
    saved = {f: getattr(torch, f) for f in factories}

    def wrap(fn):
        def inner(*a, **kw):
            if kw.get("device") == "cuda":
                kw["device"] = "cpu"
            return fn(*a, **kw)
        return inner
    for f in factories:
        setattr(torch, f, wrap(saved[f]))
    sys.path.insert(0, REF)
    try:
        import go  # the reference module
        yield go, saved
    finally:
        sys.path.remove(REF)
        for f in factories:
            setattr(torch, f, saved[f])
        for k, v in saved_mods.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v


def make_objective_fixtures():
    import torch
    with reference_go_on_cpu() as (go, saved):
        for name in cases.OBJECTIVE_CASES:
            c = cases.objective_case(name)
            chans = {k: torch.from_numpy(v) for k, v in c["channels"].items()}
            ms_list = [go.Metasurface(None, None, None, None, None, c["max_phase_deg"])
                       for _ in range(c["n_ms"])]
            model = go.Model(name, channels=chans, ms_list=ms_list,
                             max_ms_reflex=c["max_ms_reflex"], code_num=c["code_num"], w=c["w"])
            with torch.no_grad():
                model.antenna_theta.copy_(torch.from_numpy(c["theta"]))
                for i in range(c["n_ms"]):
                    model.ms_theta[i].copy_(torch.from_numpy(c["phi"][i]))
            mask_box = {}
            real_rand = torch.rand  # the device-redirecting wrapper

            def rand_hook(*a, **kw):
                out = real_rand(*a, **kw)
                mask_box["r"] = out.clone()
                return out
            torch.manual_seed(c["seed"])
            torch.rand = rand_hook
            try:
                loss = model.forward()
            finally:
                torch.rand = real_rand
            for p in model.parameters():
                p.grad = None
            loss.backward()
            drop = (mask_box["r"] < 0.1).numpy()
            out = dict(loss=np.float64(loss.item()), drop=drop,
                       recv_amp=model.result.numpy(), cap=model.cap.numpy(),
                       grad_theta=model.antenna_theta.grad.numpy())
            for i in range(c["n_ms"]):
                g = model.ms_theta[i].grad
                out[f"grad_phi{i}"] = (g.numpy() if g is not None
                                       else np.zeros_like(c["phi"][i]))
            out["input_sha"] = np.array(digest(*[c["channels"][k] for k in sorted(c["channels"])],
                                               c["theta"], *c["phi"]))
            np.savez_compressed(os.path.join(HERE, f"obj_{name}.npz"), **out)
            print(name, "loss", loss.item(), "dropped rows", int(drop.sum()))


def make_postprocess_fixtures():
    """go.Model.postprocess (go.py:89-97) on every objective case: the code
    phases rounded to pi/2 steps, the metasurface phases reduced modulo
    max_phase, then forward (go.py:159-245): the quantised parameters,
    Model.result, Model.max_code_ids and the loss, with the dropout draw."""
    import torch
    with reference_go_on_cpu() as (go, saved):
        for name in cases.OBJECTIVE_CASES:
            c = cases.objective_case(name)
            chans = {k: torch.from_numpy(v) for k, v in c["channels"].items()}
            ms_list = [go.Metasurface(None, None, None, None, None, c["max_phase_deg"])
                       for _ in range(c["n_ms"])]
            model = go.Model(name, channels=chans, ms_list=ms_list,
                             max_ms_reflex=c["max_ms_reflex"], code_num=c["code_num"], w=c["w"])
            with torch.no_grad():
                model.antenna_theta.copy_(torch.from_numpy(c["theta"]))
                for i in range(c["n_ms"]):
                    model.ms_theta[i].copy_(torch.from_numpy(c["phi"][i]) * 3.0)
            box = {}
            real_rand = torch.rand

            def rand_hook(*a, **kw):
                out = real_rand(*a, **kw)
                box["r"] = out.clone()
                return out
            torch.manual_seed(c["seed"] + 50)
            torch.rand = rand_hook
            try:
                model.postprocess()
            finally:
                torch.rand = real_rand
            out = dict(theta_post=model.antenna_theta.detach().numpy(), rand=box["r"].numpy(),
                       result=model.result.numpy(), max_code_ids=model.max_code_ids.numpy(),
                       loss=np.float64(model.loss.item() if hasattr(model, "loss")
                                       else model.forward().item()))
            for i in range(c["n_ms"]):
                out[f"phi_in{i}"] = (torch.from_numpy(c["phi"][i]) * 3.0).numpy()
                out[f"phi_post{i}"] = model.ms_theta[i].detach().numpy()
            np.savez_compressed(os.path.join(HERE, f"post_{name}.npz"), **out)
            print("postprocess", name, "loss", float(out["loss"]))


# ------------------------------------------------------------- geometry
def geometry_inputs():
    """Seeded inputs of the geometry helpers (go.py:248-512, 1309-1338)."""
    rng = np.random.Generator(np.random.PCG64(11))

    def unit(v):
        v = np.asarray(v, np.float64)
        return (v / np.linalg.norm(v)).tolist()

    def frame():
        k = np.array(unit(rng.normal(size=3)))
        i = rng.normal(size=3)
        i = i - (i @ k) * k
        return unit(k), unit(i)
    dirs = []
    for n in range(40):
        up = unit(rng.normal(size=3))
        pol = unit(rng.normal(size=3))
        th, ph = float(rng.uniform(-90, 90)), float(rng.uniform(0, 360))
        if n % 2:
            dirs.append((th / 180 * np.pi, ph / 180 * np.pi, up, pol, "rad"))
        else:
            dirs.append((th, ph, up, pol, "deg"))
    mats = []
    for size, spacing in (((3, 5), 0.0025), ((4, 4), 0.1), ((1, 6), 0.05), ((7, 2), 0.3)):
        k, i = frame()
        mats.append((rng.uniform(-5, 5, 3).tolist(), k, i, size, spacing))
    mss = []
    for size, spacing, th in (((4, 6), 0.0025, 0.001), ((3, 3), 0.2, 0.01), ((8, 5), 0.01, 0.002)):
        k, i = frame()
        mss.append((rng.uniform(-5, 5, 3).tolist(), k, i, size, spacing, th))
    walls = []
    for _ in range(6):
        ul = rng.uniform(-5, 5, 3)
        dl = ul + rng.uniform(-3, 3, 3)
        dr = dl + rng.uniform(-3, 3, 3)
        walls.append(([ul.tolist(), dl.tolist(), dr.tolist()],
                      (float(rng.uniform(0, 1)), float(rng.uniform(0, 1)))))
    ends = [([0.0, 1.0, 5], [2.0, 3.0, 4], 1.5), (0.5, [-1.0, 1.0, 3], [0.0, 2.0, 6]),
            ([1.0, 2.0, 3], 0.25, [3.0, 1.0, 4])]
    boxes = [([1.0, 2.0, 0.5], 0.2, 0.2, 1.5), ([-3.0, 0.5, 1.0], 0.7, 1.3, 0.4),
             ([0.0, 0.0, 0.0], 2.0, 1.0, 3.0)]
    return dict(dirs=dirs, mats=mats, mss=mss, walls=walls, ends=ends, boxes=boxes)


def write_scene_text_files(folder):
    """Seeded ap.txt, door.txt and wall.txt in the reference's formats
    (go.py:533-620): ap = centre line + direction line; a door = 3 vertex
    lines + a 0/1 swing line; a wall = a name line + 3 vertex lines."""
    rng = np.random.Generator(np.random.PCG64(12))
    fmt = lambda v: " ".join(f"{x:.6f}" for x in v)
    with open(os.path.join(folder, "ap.txt"), "w") as f:
        f.write(fmt(rng.uniform(0, 10, 3)) + "\n" + fmt(rng.normal(size=3)) + "\n")
    with open(os.path.join(folder, "door.txt"), "w") as f:
        for d in range(3):
            base = rng.uniform(0, 10, 3)
            base[2] = 0.0
            f.write(fmt(base + [0, 0, 2.1]) + "\n" + fmt(base) + "\n")
            f.write(fmt(base + np.append(rng.uniform(-1, 1, 2), 0.0)) + "\n" + f"{d % 2}\n")
    with open(os.path.join(folder, "wall.txt"), "w") as f:
        for w in range(4):
            f.write(f"wall{w}\n")
            for _ in range(3):
                f.write(fmt(rng.uniform(-5, 5, 3)) + "\n")


DOOR_ANGLES = (0.0, 0.3, -1.2)


def make_geometry_fixtures():
    import tempfile
    g = geometry_inputs()
    out = {}
    with reference_go_on_cpu() as (go, _):
        with tempfile.TemporaryDirectory() as d:
            write_scene_text_files(d)
            c, k = go.get_ap(d)
            out["ap"] = np.asarray([c, k], np.float64)
            for n, ang in enumerate(DOOR_ANGLES):
                out[f"doors{n}"] = np.asarray(go.get_doors(d, ang), np.float64)
            out["walls"] = np.asarray(go.get_walls(d), np.float64)
        for n, (th, ph, up, pol, u) in enumerate(g["dirs"]):
            out[f"dir{n}"] = go.gen_direction_from_angle(th, ph, up, pol, unit=u).numpy()
        for n, (c, k, i, size, sp) in enumerate(g["mats"]):
            out[f"mat{n}"] = go.gen_pos_matrix(c, k, i, size, sp).numpy()
        for n, (c, k, i, size, sp, th) in enumerate(g["mss"]):
            pos, bh, kd = go.gen_ms(c, k, i, size, sp, th)
            out[f"ms{n}_pos"] = pos.numpy()
            out[f"ms{n}_bh"] = np.asarray(bh, np.float32)
            out[f"ms{n}_k"] = kd.numpy()
        for n, (w, ij) in enumerate(g["walls"]):
            v, kd, idir = go.gen_sth_from_wall(w, ij)
            out[f"wall{n}"] = np.stack([v.numpy(), kd.numpy(), idir.numpy()])
        for n, (x, y, z) in enumerate(g["ends"]):
            out[f"end{n}"] = go.gen_pos_from_endpoint(x, y, z).numpy()
        for n, (c, xl, yl, zl) in enumerate(g["boxes"]):
            out[f"box{n}"] = np.asarray(go.create_vertex_buffer(c, xl, yl, zl), np.float32)
    np.savez_compressed(os.path.join(HERE, "geometry_ref.npz"), **out)
    print("geometry fixtures written:", len(out))


# ------------------------------------------------- the reference's scene
def make_reference_scene_fixtures():
    """go.py's own build_channels on the reference scene stl/4321, reduced
    (cases.reference_scene_setup: 2x2 AP, 20x18 Rx, two metasurfaces, a
    door and a reflector quad, 3 reflections, go.py's 100 x 100 launch): the
    reference's ingest (go.py:679-737) and channel-set logic
    (go.py:1135-1247) run as written, its OptiX op replaced by the
    reference's device programs on the CPU (oracle/ref_harness).  Saved: the
    scene folder's files in this folder's listdir order, the inputs, the
    ingest of every trace (full arrays for the first, sha256 for all) and per
    trace H, counters and the ordered path list."""
    import torch
    folder = os.path.join(REF, *cases.REF_SCENE.split("/"))
    lam = 3e8 / 60e9
    traces = []

    def op(result, src, dst, src_buffer, dst_buffer, scene_buffer, mat, spl, lx, ly, wave_len,
           L, reserve, mat_prop, src_dir, dst_dir, log_level, sbp, dbp, gs, src_r, dst_r):
        params = dict(samples_per_launch=int(spl), launch_x=int(lx), launch_y=int(ly),
                      wave_len=float(wave_len), max_reflection=int(L), reserve_size=int(reserve),
                      src_bptype=int(sbp), dst_bptype=int(dbp), dst_gridsize=int(gs),
                      src_r=float(src_r), dst_r=float(dst_r),
                      src_dir=[float(x) for x in src_dir], dst_dir=[float(x) for x in dst_dir])
        sb = scene_buffer.numpy().astype(np.float32)
        H, st, paths = oracle.ref_trace_channel(sb.reshape(-1, 9), mat.numpy(), mat_prop.numpy(),
                                                src.numpy(), dst.numpy(), params,
                                                src_box=src_buffer.numpy(),
                                                dst_box=dst_buffer.numpy())
        result[..., 0] += torch.from_numpy(np.ascontiguousarray(H.real))
        result[..., 1] += torch.from_numpy(np.ascontiguousarray(H.imag))
        traces.append(dict(params=params, H=H, paths=paths,
                           stats=np.array([st[k] for k in cases.STAT_KEYS], np.int64),
                           ingest_sha=digest(sb, mat.numpy().astype(np.int32),
                                             mat_prop.numpy().astype(np.float32)),
                           n_tri=sb.shape[0] // 3,
                           scene=(sb, mat.numpy().astype(np.int32),
                                  mat_prop.numpy().astype(np.float32))))
        print("  trace", len(traces), st, flush=True)

    with reference_go_on_cpu() as (go, _):
        setup = cases.reference_scene_setup(go, folder, lam)
        saved_ops = torch.ops
        torch.ops = types.SimpleNamespace(
            pathtrace=types.SimpleNamespace(torch_launch_pathtrace=op))
        try:
            ch = go.build_channels(setup["src"], setup["dst"], setup["ms_list"], setup["ap_dir"],
                                   folder, lam, cases.REF_SCENE_L,
                                   reflector_buffer=setup["reflector"],
                                   door_buffer=setup["door"])
        finally:
            torch.ops = saved_ops
    keys = list(ch.keys())
    assert len(keys) == len(traces)
    names = [f for f in os.listdir(folder) if f.endswith(".stl")]
    blocks = [StubMesh.from_file(os.path.join(folder, f)).vectors for f in names]
    with open(os.path.join(folder, "mat.txt")) as f:
        mat_txt = f.read()
    with open(os.path.join(folder, "wall.txt")) as f:
        wall_txt = f.read()
    out = dict(stl_names=np.array(names), stl_counts=np.array([len(b) for b in blocks]),
               stl_tris=np.concatenate(blocks, 0), mat_txt=np.array(mat_txt),
               wall_txt=np.array(wall_txt), keys=np.array(keys),
               src=setup["src"].numpy(), dst=setup["dst"].numpy(),
               ap_dir=setup["ap_dir"].numpy(),
               door=np.asarray(setup["door"], np.float32),
               reflector=np.asarray(setup["reflector"], np.float32))
    for i, m in enumerate(setup["ms_list"]):
        out[f"ms{i}_pos"] = m.pos.numpy()
        out[f"ms{i}_send"] = m.send_dir.numpy()
        out[f"ms{i}_recv"] = m.recv_dir.numpy()
        out[f"ms{i}_blackhole"] = np.asarray(m.blackhole, np.float32)
        out[f"ms{i}_size"] = np.asarray(m.size)
    sb, mt, mp = traces[0]["scene"]
    out["scene0_buffer"], out["scene0_mat"], out["scene0_mat_prop"] = sb, mt, mp
    for k, t in zip(keys, traces):
        tag = k.replace("{", "").replace("}", "")
        out[f"{tag}_H"] = t["H"]
        out[f"{tag}_paths"] = t["paths"]
        out[f"{tag}_stats"] = t["stats"]
        out[f"{tag}_ingest_sha"] = np.array(t["ingest_sha"])
        out[f"{tag}_n_tri"] = np.array(t["n_tri"])
        out[f"{tag}_params"] = np.array(json.dumps(t["params"]))
        assert np.array_equal(ch[k].numpy(), t["H"])
    np.savez_compressed(os.path.join(HERE, "ref_scene_4321.npz"), **out)
    print("reference-scene fixtures written:", keys)


if __name__ == "__main__":
    if not REF or not oracle.ref_available():
        raise SystemExit("AMS_REFERENCE_ROOT does not name the reference tree; "
                         "fixtures cannot be regenerated")
    if sys.argv[1:] == ["postprocess"]:
        make_postprocess_fixtures()
        raise SystemExit(0)
    if sys.argv[1:] == ["ref_scene"]:
        make_reference_scene_fixtures()
        raise SystemExit(0)
    if len(sys.argv) > 1:  # regenerate the named channel fixtures only
        make_channel_fixtures(sys.argv[1:])
        raise SystemExit(0)
    make_unit_fixtures()
    make_channel_fixtures()
    make_objective_fixtures()
    make_postprocess_fixtures()
    make_geometry_fixtures()
    make_reference_scene_fixtures()
