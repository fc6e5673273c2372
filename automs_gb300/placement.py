"""Metasurface placement study: ray-traced gain maps, surrogate screening and
simulated annealing.

Reference behaviour: one NNI trial (physical_exp_nni_model.py:7-149) places a
metasurface on a wall (gen_sth_from_wall + gen_ms, go.py:388-477), builds the
AP->Rx, AP->MS and MS->Rx channels (build_channels, go.py:1135-1247),
optimises the phase map (optimize_model, go.py:296-336) and reports a loss;
NNI's annealer proposes the next placement (physical_exp_nni_main.py:11-24).

Here a trial is `PlacementStudy.evaluate`: the same three traces on the GPU,
a phase-map optimisation on the CUDA objective, and the coverage gain (dB,
with the optimised metasurface minus without) pooled to a coarse map.  The
surrogate MLP (surrogate.py) learns descriptor -> gain map from such trials;
`screened_anneal` lets it rank annealing candidates so that the tracer only
judges the best few.
"""
import math
import time

import numpy as np
import torch

from . import objective, scenes, tracer

N_PARAMS = 8
N_OCC = 64


class PlacementStudy:
    """A seeded room with an AP and an Rx grid; placements on 3 walls."""

    def __init__(self, seed=0, rx=(64, 64), launch=250, max_reflection=2, pool=4,
                 opt_steps=30, n_boxes=12, sizes=(8, 24)):
        self.seed = seed
        self.lam = scenes.WAVE_LEN_60GHZ
        self.room = (12.0, 8.0, 3.0)
        self.ap_pos = (6.0, 0.5, 2.5)
        self.tris, self.mat, self.mat_prop = scenes.shoebox_scene(
            n_boxes, room=self.room, box_tess=1, seed=seed, keep_clear=[self.ap_pos])
        self.src = scenes.ula(self.ap_pos, (1, 0, 0), 16, self.lam / 2)
        self.dst = scenes.rx_grid(0.25, 11.75, rx[0], 0.25, 7.75, rx[1], 1.5)
        self.rx = rx
        self.pool = pool
        self.launch = launch
        self.L = max_reflection
        self.opt_steps = opt_steps
        self.sizes = sizes
        # walls: (origin of the u axis, u direction, inward normal, length)
        X, Y, Z = self.room
        self.walls = [
            (np.array([0.0, Y, 0.0]), np.array([1.0, 0.0, 0.0]), np.array([0.0, -1.0, 0.0]), X),
            (np.array([0.0, 0.0, 0.0]), np.array([0.0, 1.0, 0.0]), np.array([1.0, 0.0, 0.0]), Y),
            (np.array([X, 0.0, 0.0]), np.array([0.0, 1.0, 0.0]), np.array([-1.0, 0.0, 0.0]), Y),
        ]
        self.occupancy = self._occupancy()
        wv = np.ones(16, np.complex64) / 4.0
        self.W = torch.as_tensor(wv[None], device="cuda")
        self.scene = tracer.Scene(self.tris, self.mat, self.mat_prop)
        H0, _ = self._trace(self.scene, self.src, self.dst, 2, 0, (0, 1, 0), (0, 0, 0))
        self.db0 = self._coverage(H0)

    # ------------------------------------------------------------ helpers
    def _occupancy(self):
        X, Y, _ = self.room
        occ = np.zeros((8, 8))
        t = self.tris.reshape(-1, 3, 3)
        lo = t.min(1)
        hi = t.max(1)
        boxes = self.mat >= 3
        for i in range(8):
            for j in range(8):
                cx0, cx1 = i * X / 8, (i + 1) * X / 8
                cy0, cy1 = j * Y / 8, (j + 1) * Y / 8
                ox = np.clip(np.minimum(hi[boxes, 0], cx1) - np.maximum(lo[boxes, 0], cx0), 0, None)
                oy = np.clip(np.minimum(hi[boxes, 1], cy1) - np.maximum(lo[boxes, 1], cy0), 0, None)
                occ[i, j] = min(1.0, float((ox * oy).sum()) / (X * Y / 64) / 12.0)
        return occ.reshape(-1).astype(np.float32)

    def _params(self, launch):
        return tracer.make_params(launch, launch, self.lam, self.L, 100)

    def _trace(self, scene, src, dst, sbp, dbp, sdir, ddir):
        p = tracer.make_params(self.launch, self.launch, self.lam, self.L, 100, sbp, dbp, 5,
                               0.5e-5, 0.06, sdir, ddir)
        res, st = scene.trace(src, dst, p)
        return torch.complex(res[..., 0], res[..., 1]), st

    def _coverage(self, H):
        y = (self.W @ H).abs()[0]
        db = 20 * torch.log10(y + 1e-12)
        n0, n1 = self.rx
        g = db.reshape(n0 // self.pool, self.pool, n1 // self.pool, self.pool).mean((1, 3))
        return g.reshape(-1)

    def ms_geometry(self, p):
        """p = (wall, u, v, size): wall index, position along the wall and
        height as fractions, side length in elements (lambda/2 pitch)."""
        wall, u, v, n = int(p[0]), float(p[1]), float(p[2]), int(p[3])
        org, ud, nrm, length = self.walls[wall]
        up = np.array([0.0, 0.0, 1.0])
        center = org + ud * (u * length) + up * (0.3 + v * 2.4) + nrm * 1e-3
        pitch = self.lam / 2
        k = np.arange(n) - (n - 1) / 2
        side = np.cross(nrm, up)
        pos = (center[None, None, :] - k[:, None, None] * pitch * up[None, None, :]
               + k[None, :, None] * pitch * side[None, None, :]).astype(np.float32)
        h = n / 2 * pitch + 1e-3
        c = center - nrm * 5e-4
        a, b = up * h, side * h
        quad = np.array([[c - a - b, c - a + b, c + a - b], [c + a - b, c + a + b, c - a + b]],
                        np.float32)
        return pos, quad, nrm.astype(np.float32)

    def descriptor(self, p):
        wall, u, v, n = int(p[0]), float(p[1]), float(p[2]), int(p[3])
        lo, hi = self.sizes
        d = np.zeros(N_PARAMS, np.float32)
        d[wall] = 1.0
        d[3], d[4] = u, v
        d[5] = (n - lo) / max(1, hi - lo)
        d[6], d[7] = math.sin(math.pi * u), math.cos(math.pi * u)
        return np.concatenate([d, self.occupancy])

    def random_params(self, rng):
        lo, hi = self.sizes
        return (int(rng.integers(0, 3)), float(rng.uniform(0.1, 0.9)), float(rng.uniform(0.1, 0.9)),
                int(rng.integers(lo // 8, hi // 8 + 1) * 8))

    # ---------------------------------------------------------- one trial
    def evaluate(self, p, return_detail=False):
        """Ray-trace + optimise one placement; returns the pooled gain map (dB)."""
        pos, quad, nrm = self.ms_geometry(p)
        tris = np.concatenate([self.tris, quad], 0)
        mat = np.concatenate([self.mat, np.full(2, self.mat_prop.shape[0], np.int32)])
        mp = np.concatenate([self.mat_prop, np.zeros((1, 19), np.float32)], 0)  # blackhole
        sc = tracer.Scene(tris, mat, mp)
        Hd, _ = self._trace(sc, self.src, self.dst, 2, 0, (0, 1, 0), (0, 0, 0))
        sc.close()
        Ha, _ = self._trace(self.scene, self.src, pos, 2, 1, (0, 1, 0), nrm)
        Hr, _ = self._trace(self.scene, pos, self.dst, 1, 0, nrm, (0, 0, 0))
        M = pos.shape[0] * pos.shape[1]
        phi = torch.zeros(M, device="cuda", requires_grad=True)
        opt = torch.optim.Adam([phi], lr=0.3)
        R = Hd.shape[1]
        for _ in range(self.opt_steps):
            loss = objective.capacity_objective(self.W, Hd, Ha, Hr, phi, 2 * math.pi, 1.0 / R)
            loss.backward()
            opt.step()
            opt.zero_grad()
        with torch.no_grad():
            H = Hd + (Ha * torch.exp(1j * phi)[None, :]) @ Hr
            gain = self._coverage(H) - self.db0
        if return_detail:
            return gain, dict(H=H, phi=phi.detach())
        return gain

    def dataset(self, n, seed=0, log=None):
        rng = np.random.Generator(np.random.PCG64(seed))
        X, Y, P = [], [], []
        t0 = time.time()
        for i in range(n):
            p = self.random_params(rng)
            X.append(self.descriptor(p))
            Y.append(self.evaluate(p).float().cpu().numpy())
            P.append(p)
            if log and (i + 1) % 100 == 0:
                log(f"{i + 1}/{n} samples, {time.time() - t0:.1f}s")
        return np.stack(X), np.stack(Y), P


class TwoRoomStudy:
    """Metasurface placement for a non-line-of-sight room: a pool of seeded
    two-room floors (scenes.tworoom_scene); the AP (16-element ULA, 2.5 m,
    facing +x) stands in room A 1.5 m before the door gap, the Rx grid covers
    room B at 1.5 m, and the metasurface hangs on one of room A's three
    other walls, facing into room A, where the AP lights it.  Most of room B
    sees the AP only through the door at a narrow angle; a metasurface that
    also sees through the door relays power into the rest of it, the
    situation of the reference's trial (a metasurface lighting the area a
    wall-mounted AP covers poorly, physical_exp_nni_model.py:26-87).

    With max_reflection = 1 most of room B has no path from the AP at all
    (57% of the cells of the 16 floors of seed 3) and sits at the coverage
    floor, so a placement that relays through the door gains tens of dB
    there; with 2 the AP reaches most cells within two bounces and the
    gains are small.

    A placement is p = (scene, wall, u, v, n): the scene of the pool, the
    wall (0: back wall x = 0, 1: side y = 0, 2: side y = d, both over room
    A), the position along it and the height as fractions, and the side in
    elements (lambda/2 pitch).  Its descriptor is 8 placement numbers and the scene's
    64-value code (8 x 8 cells over the floor: the share of each cell taken
    by walls and boxes, door gap included), so the code varies per sample."""

    def __init__(self, n_scenes=16, seed=0, rx=(64, 64), launch=250, max_reflection=2,
                 opt_steps=12, sizes=(16, 48)):
        self.lam = scenes.WAVE_LEN_60GHZ
        self.rx = rx
        self.pool = 1
        self.launch = launch
        self.L = max_reflection
        self.opt_steps = opt_steps
        self.sizes = sizes
        wv = np.ones(16, np.complex64) / 4.0
        self.W = torch.as_tensor(wv[None], device="cuda")
        self.scenes = []
        for k in range(n_scenes):
            tris, mat, mp, g = scenes.tworoom_scene(seed * 1000 + k)
            a, b, d = g["a"], g["b"], g["d"]
            ap = (a - 1.5, g["y_door"], 2.5)
            src = scenes.ula(ap, (0, 1, 0), 16, self.lam / 2)
            dst = scenes.rx_grid(a + 0.25, a + b - 0.25, rx[0], 0.25, d - 0.25, rx[1], 1.5)
            sc = tracer.Scene(tris, mat, mp)
            entry = dict(tris=tris, mat=mat, mat_prop=mp, geo=g, src=src, dst=dst, scene=sc,
                         code=self._code(g))
            H0, _ = self._trace(sc, src, dst, 2, 0, (1, 0, 0), (0, 0, 0))
            entry["db0"] = self._coverage(H0)
            self.scenes.append(entry)

    # ------------------------------------------------------------ helpers
    @staticmethod
    def _code(g):
        a, b, d, yd = g["a"], g["b"], g["d"], g["y_door"]
        X = a + b
        occ = np.zeros((8, 8))
        rects = [((lo[0], lo[1]), (hi[0], hi[1])) for lo, hi in g["boxes"]]
        t = 0.15  # walls as strips
        rects += [((0, 0), (X, t)), ((0, d - t), (X, d)), ((0, 0), (t, d)), ((X - t, 0), (X, d)),
                  ((a - t / 2, 0), (a + t / 2, yd - g["door_half"])),
                  ((a - t / 2, yd + g["door_half"]), (a + t / 2, d))]
        for i in range(8):
            for j in range(8):
                cx0, cx1, cy0, cy1 = i * X / 8, (i + 1) * X / 8, j * d / 8, (j + 1) * d / 8
                area = 0.0
                for (x0, y0), (x1, y1) in rects:
                    area += (max(0.0, min(x1, cx1) - max(x0, cx0))
                             * max(0.0, min(y1, cy1) - max(y0, cy0)))
                occ[i, j] = min(1.0, 8.0 * area / ((X / 8) * (d / 8)))
        return occ.reshape(-1).astype(np.float32)

    def _trace(self, scene, src, dst, sbp, dbp, sdir, ddir):
        p = tracer.make_params(self.launch, self.launch, self.lam, self.L, 100, sbp, dbp, 5,
                               0.5e-5, 0.06, sdir, ddir)
        res, st = scene.trace(src, dst, p)
        return torch.complex(res[..., 0], res[..., 1]), st

    # coverage floor (dB): an Rx without paths counts as this, so a gain is
    # the rise above the floor, not above -240 dB
    FLOOR_DB = -110.0

    def _coverage(self, H):
        db = 20 * torch.log10((self.W @ H).abs()[0] + 1e-12)
        return db.clamp_min(self.FLOOR_DB).reshape(-1)

    def ms_geometry(self, p):
        k, wall, u, v, n = int(p[0]), int(p[1]), float(p[2]), float(p[3]), int(p[4])
        g = self.scenes[k]["geo"]
        a, b, d = g["a"], g["b"], g["d"]
        if wall == 0:
            center, nrm = np.array([0.0, d * (0.05 + 0.9 * u), 0.0]), np.array([1.0, 0, 0])
        elif wall == 1:
            center, nrm = np.array([a * (0.05 + 0.9 * u), 0.0, 0.0]), np.array([0, 1.0, 0])
        else:
            center, nrm = np.array([a * (0.05 + 0.9 * u), d, 0.0]), np.array([0, -1.0, 0])
        center[2] = 0.5 + 2.0 * v
        pos, quad, kdir = scenes.metasurface(center, nrm, (0, 0, -1), n, self.lam / 2)
        return pos, quad, kdir

    def descriptor(self, p):
        """8 placement numbers in the scene's frame -- the metasurface
        centre's offset from the AP (x, y, z over 10 m), its normal (x, y),
        its side (0..1 over the sizes), and where the line from that centre
        to the centre of room B crosses the wall between the rooms: its
        offset from the door gap's centre over the gap's half width, and its
        height over the gap's height (both within 1: the metasurface looks
        into room B through the door; both clipped to [-3, 3]) -- then the
        scene's 64-value code."""
        k, n = int(p[0]), int(p[4])
        e = self.scenes[k]
        g = e["geo"]
        lo, hi = self.sizes
        pos, _, nrm = self.ms_geometry(p)
        c = pos.reshape(-1, 3).mean(0).astype(np.float64)
        ap = e["src"].reshape(-1, 3).mean(0).astype(np.float64)
        rb = np.array([g["a"] + g["b"] / 2, g["d"] / 2, 1.5])
        t = (g["a"] - c[0]) / (rb[0] - c[0])  # room B's centre lies beyond the wall
        y_at = c[1] + t * (rb[1] - c[1])
        z_at = c[2] + t * (rb[2] - c[2])
        dsc = np.array([(c[0] - ap[0]) / 10, (c[1] - ap[1]) / 10, (c[2] - ap[2]) / 10,
                        float(nrm[0]), float(nrm[1]), (n - lo) / max(1, hi - lo),
                        float(np.clip((y_at - g["y_door"]) / g["door_half"], -3, 3)),
                        float(np.clip(z_at / 2.1, -3, 3))], np.float32)
        return np.concatenate([dsc, e["code"]])

    def random_params(self, rng, scene=None):
        lo, hi = self.sizes
        k = int(rng.integers(0, len(self.scenes))) if scene is None else int(scene)
        return (k, int(rng.integers(0, 3)), float(rng.uniform(0.05, 0.95)),
                float(rng.uniform(0.05, 0.95)), int(rng.integers(lo // 8, hi // 8 + 1) * 8))

    def neighbour(self, p, rng):
        """Annealing move within p's scene: another wall with probability
        0.1, (u, v) by N(0, 0.08) clipped to [0.05, 0.95], the side by +-8
        with probability 0.2 within the sizes."""
        k, w, u, v, n = p
        if rng.random() < 0.1:
            w = int(rng.integers(0, 3))
        u = float(np.clip(u + rng.normal(0, 0.08), 0.05, 0.95))
        v = float(np.clip(v + rng.normal(0, 0.08), 0.05, 0.95))
        if rng.random() < 0.2:
            lo, hi = self.sizes
            n = int(np.clip(n + 8 * rng.choice([-1, 1]), lo, hi))
        return (k, w, u, v, n)

    # ---------------------------------------------------------- one trial
    def evaluate(self, p, return_detail=False):
        """Trace + optimise one placement; returns its gain map (dB over the
        Rx grid, with the optimised metasurface minus without)."""
        return self._evaluate_on(p, self.scenes[int(p[0])]["scene"], None, return_detail)

    def _evaluate_on(self, p, scene, obj_lock, return_detail=False):
        e = self.scenes[int(p[0])]
        pos, quad, nrm = self.ms_geometry(p)
        sc = tracer.Scene(*scenes.with_blackholes(e["tris"], e["mat"], e["mat_prop"], [quad]))
        Hd, _ = self._trace(sc, e["src"], e["dst"], 2, 0, (1, 0, 0), (0, 0, 0))
        sc.close()
        Ha, _ = self._trace(scene, e["src"], pos, 2, 1, (1, 0, 0), nrm)
        Hr, _ = self._trace(scene, pos, e["dst"], 1, 0, nrm, (0, 0, 0))
        M = pos.shape[0] * pos.shape[1]
        R = Hd.shape[1]
        # the objective's scratch is per device: concurrent placements run
        # their optimisation one at a time, each finished before the next
        if obj_lock is not None:
            obj_lock.acquire()
        try:
            phi = torch.zeros(M, device="cuda", requires_grad=True)
            opt = torch.optim.Adam([phi], lr=0.3)
            for _ in range(self.opt_steps):
                loss = objective.capacity_objective(self.W, Hd, Ha, Hr, phi, 2 * math.pi, 1.0 / R)
                loss.backward()
                opt.step()
                opt.zero_grad()
            with torch.no_grad():
                _, recv = objective.capacity_objective(self.W, Hd, Ha, Hr, phi.detach(),
                                                       2 * math.pi, 1.0 / R, return_recv=True)
                db = (20 * torch.log10(recv[0] + 1e-12)).clamp_min(self.FLOOR_DB).reshape(-1)
                gain = db - e["db0"]
            if obj_lock is not None:
                torch.cuda.current_stream().synchronize()
        finally:
            if obj_lock is not None:
                obj_lock.release()
        if return_detail:
            return gain, dict(phi=phi.detach())
        return gain

    def evaluate_many(self, ps, workers=4):
        """evaluate() of several placements at once, results equal to one at
        a time: `workers` host threads, each with its own CUDA stream and
        its own scene handles, so that one placement's traces (and their
        flood-fill round trips) overlap the others'; the optimisation steps
        of one placement at a time.  The plain annealing loop cannot do
        this (each move waits for the last one's result); a screened search
        knows the placements it will judge in advance."""
        import concurrent.futures as cf
        import threading
        local = threading.local()
        made, lock, obj_lock = [], threading.Lock(), threading.Lock()

        def work(p):
            if not hasattr(local, "stream"):
                local.stream, local.scenes = torch.cuda.Stream(), {}
            k = int(p[0])
            with torch.cuda.stream(local.stream):
                if k not in local.scenes:
                    e = self.scenes[k]
                    local.scenes[k] = tracer.Scene(e["tris"], e["mat"], e["mat_prop"])
                    with lock:
                        made.append(local.scenes[k])
                g = self._evaluate_on(p, local.scenes[k], obj_lock)
                local.stream.synchronize()
                return g

        torch.cuda.synchronize()
        try:
            with cf.ThreadPoolExecutor(max_workers=workers) as ex:
                out = list(ex.map(work, ps))
        finally:
            torch.cuda.synchronize()
            for s_ in made:
                s_.close()
        return out

    def dataset(self, n, seed=0, log=None, scene=None, workers=1):
        """n seeded random placements with their descriptors and traced gain
        maps; with workers > 1 traced by evaluate_many (same results)."""
        rng = np.random.Generator(np.random.PCG64(seed))
        P = [self.random_params(rng, scene) for _ in range(n)]
        X = [self.descriptor(p) for p in P]
        if workers > 1:
            Y = [g.float().cpu().numpy() for g in self.evaluate_many(P, workers)]
        else:
            Y = []
            for i, p in enumerate(P):
                Y.append(self.evaluate(p).float().cpu().numpy())
                if log and (i + 1) % 200 == 0:
                    log(f"{i + 1}/{n} samples")
        return np.stack(X), np.stack(Y), P

    def close(self):
        for e in self.scenes:
            e["scene"].close()


def score(gain):
    """Placement figure of merit: mean pooled coverage gain (dB)."""
    return gain.mean(-1)


def anneal_candidates(study, n, rng, surrogate=None, t0=1.0, t1=0.02, device="cuda",
                      start=None):
    """Simulated-annealing chain over placements (the NNI Anneal tuner's role,
    physical_exp_nni_main.py:11-29), from `start` or a random placement.
    Moves: study.neighbour when the study has one, else another wall with
    probability 0.1, the position (u, v) by N(0, 0.08) clipped to [0.1, 0.9],
    the size by +-8 with probability 0.2 within study.sizes.  With a
    surrogate (a callable on descriptors placed on `device`), moves are
    accepted on its predicted score by the Metropolis rule at a temperature
    falling geometrically from t0 to t1; every visited placement is
    returned."""
    cur = study.random_params(rng) if start is None else start
    visited = [cur]
    cur_s = None
    batch = 256
    props = []
    while len(visited) < n:
        # propose a batch of neighbours, score them together
        props = []
        for _ in range(batch):
            if hasattr(study, "neighbour"):
                props.append(study.neighbour(cur, rng))
                continue
            w, u, v, s = cur
            if rng.random() < 0.1:
                w = int(rng.integers(0, 3))
            u = float(np.clip(u + rng.normal(0, 0.08), 0.1, 0.9))
            v = float(np.clip(v + rng.normal(0, 0.08), 0.1, 0.9))
            if rng.random() < 0.2:
                lo, hi = study.sizes
                s = int(np.clip(s + 8 * rng.choice([-1, 1]), lo, hi))
            props.append((w, u, v, s))
        if surrogate is not None:
            X = torch.as_tensor(np.stack([study.descriptor(q) for q in props]), device=device)
            sc = score(surrogate(X)).cpu().numpy()
        else:
            sc = rng.normal(size=len(props))
        for q, s_ in zip(props, sc):
            T = t0 * (t1 / t0) ** (len(visited) / n)
            if cur_s is None or s_ > cur_s or rng.random() < math.exp((s_ - cur_s) / T):
                cur, cur_s = q, s_
            visited.append(q)
            if len(visited) >= n:
                break
    return visited[:n]


def anneal_traced(study, n, rng, start, t0=1.0, t1=0.02):
    """The plain annealing loop: the same Metropolis chain with every move
    judged by the tracer (study.evaluate), as the reference's tuner judges
    each trial by running it.  Returns the visited placements, their traced
    scores and the wall time."""
    torch.cuda.synchronize()
    t_start = time.perf_counter()
    cur = start
    cur_s = float(score(study.evaluate(cur)))
    seen, scores = [cur], [cur_s]
    while len(seen) < n:
        q = study.neighbour(cur, rng)
        s_ = float(score(study.evaluate(q)))
        T = t0 * (t1 / t0) ** (len(seen) / n)
        if s_ > cur_s or rng.random() < math.exp((s_ - cur_s) / T):
            cur, cur_s = q, s_
        seen.append(q)
        scores.append(s_)
    torch.cuda.synchronize()
    return seen, np.asarray(scores), time.perf_counter() - t_start


def screening_report(study, mlp, pool_params, pool_gain, top_frac=0.05, t_trial=None,
                     mlp_batch=4096):
    """Compare surrogate screening with the plain loop on a traced pool.

    pool_params / pool_gain: placements and their traced gain maps (the plain
    loop's answer).  The surrogate ranks the whole pool, the tracer judges the
    top `top_frac`; the pick is compared with the pool's true best.  Rates:
    plain = 1 / t_trial configs/s; screened = n / (t_rank + k t_trial)."""
    n = len(pool_params)
    k = max(1, int(round(top_frac * n)))
    X = torch.as_tensor(np.stack([study.descriptor(p) for p in pool_params]), device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pred = mlp(X)
    torch.cuda.synchronize()
    t_rank = time.perf_counter() - t0
    ps = score(pred).cpu().numpy()
    true = score(torch.as_tensor(pool_gain)).numpy()
    top = np.argsort(-ps)[:k]
    pick = top[np.argmax(true[top])]
    if t_trial is None:
        t0 = time.perf_counter()
        study.evaluate(pool_params[0])
        torch.cuda.synchronize()
        t_trial = time.perf_counter() - t0
    err = np.abs(pred.cpu().numpy() - pool_gain)
    return {
        "pool": n, "judged": k,
        "surrogate_median_abs_err_db": float(np.median(err)),
        "mean_predictor_median_abs_err_db": float(np.median(np.abs(pool_gain - pool_gain.mean(0)))),
        "best_true_score_db": float(true.max()), "screened_pick_score_db": float(true[pick]),
        "selection_gap_db": float(true.max() - true[pick]),
        "pick_median_cell_err_db": float(np.median(np.abs(pool_gain[pick] - pool_gain[np.argmax(true)]))),
        "t_trial_s": t_trial, "t_rank_s": t_rank,
        "plain_configs_per_s": 1.0 / t_trial,
        "screened_configs_per_s": n / (t_rank + k * t_trial),
    }


def batch_evaluate(cfg, indices=None, workers=4, opt_steps=20, lr=0.3, keep=False):
    """Batched hyper-configs (scenes.batch_config): for each placement the
    AP->Rx channel with the metasurface as a blackhole, the AP->MS and MS->Rx
    channels (build_channels, go.py:1135-1247), then opt_steps Adam steps of
    the phase map on an evaluation plan (optimize_model, go.py:296-336, with
    C = 1 and w = 1/R).

    Placements run on `workers` host threads, each with its own CUDA stream
    and scene handle, so one placement's flood-fill round trips overlap the
    others' kernels.  Returns per-placement results and the wall time.  Each
    result has the loss of the first and the last step, and ms_share: the
    power the metasurface path carries at phi = 0 over the power of the
    direct channel, summed over the Rx grid (after the timed work).  With
    keep=True a result also holds the channels, the weights and the final
    phase map (keys H, w, phi)."""
    import concurrent.futures as cf
    import threading

    from . import objective as obj
    from . import scenes as sc_mod

    if indices is None:
        indices = list(range(len(cfg["placements"])))
    src, dst = cfg["src"], cfg["dst"]
    R = dst.shape[0] * dst.shape[1]
    S = src.shape[0] * src.shape[1]
    prm = cfg["prm"]
    none = (0.0, 0.0, 0.0)
    local = threading.local()
    scenes_made = []
    lock = threading.Lock()

    def work(pi):
        if not hasattr(local, "scene"):
            local.stream = torch.cuda.Stream()
            with torch.cuda.stream(local.stream):
                local.scene = tracer.Scene(cfg["tris"], cfg["mat"], cfg["mat_prop"])
            with lock:
                scenes_made.append(local.scene)
        pl = cfg["placements"][pi]
        pos, k = pl["pos"], tuple(float(x) for x in pl["normal"])
        with torch.cuda.stream(local.stream):
            t0 = time.perf_counter()
            bh = tracer.Scene(*sc_mod.with_blackholes(cfg["tris"], cfg["mat"], cfg["mat_prop"],
                                                      [pl["blackhole"]]))
            rd, sd = bh.trace(src, dst, tracer.params_from_dict(prm(2, 0, cfg["ap_dir"], none)))
            bh.close()
            ra, sa = local.scene.trace(src, pos, tracer.params_from_dict(prm(2, 1, cfg["ap_dir"], k)))
            rr, sr = local.scene.trace(pos, dst, tracer.params_from_dict(prm(1, 0, k, none)))
            Hd, Ha, Hr = (torch.view_as_complex(x) for x in (rd, ra, rr))
            t1 = time.perf_counter()
            M = Ha.shape[1]
            plan = obj.ObjectivePlan(Hd, Ha, Hr, c_max=1)
            w = torch.ones(1, S, dtype=torch.complex64, device="cuda") / math.sqrt(S)
            phi = torch.zeros(M, device="cuda", requires_grad=True)
            opt = torch.optim.Adam([phi], lr=lr)
            first = last = None
            for _ in range(opt_steps):
                loss = obj.capacity_objective(w, Hd, Ha, Hr, phi, 2 * math.pi, 1.0 / R, plan=plan)
                loss.backward()
                opt.step()
                opt.zero_grad()
                lv = loss.detach()
                first = lv if first is None else first
                last = lv
            first_v, last_v = float(first), float(last)
            obj.check_status(plan)
            plan.close()
            local.stream.synchronize()
            t2 = time.perf_counter()
            with torch.no_grad():
                yd = (w @ Hd).abs().pow(2).sum()
                ym = ((w @ Ha) @ Hr).abs().pow(2).sum()
                share = float(ym / yd) if float(yd) > 0 else float("inf")
        out = dict(index=pi, size=pl["size"], M=M,
                   rx_paths=sd["rx_paths"] + sa["rx_paths"] + sr["rx_paths"],
                   ms_to_rx_paths=sr["rx_paths"], ap_to_ms_paths=sa["rx_paths"],
                   t_trace=t1 - t0, t_opt=t2 - t1, loss_first=first_v, loss_last=last_v,
                   ms_share=share)
        if keep:
            out.update(H=(Hd, Ha, Hr), w=w, phi=phi.detach().clone())
        return out

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        res = list(ex.map(work, indices))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    for s_ in scenes_made:
        s_.close()
    return res, wall
