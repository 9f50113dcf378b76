"""Seeded synthetic inputs of the five expansion workloads.

No benchmark suite or primitive set of the reference ships with it (the
dynomotions submodule and the dynobench environments are empty), so every
input is generated here from a recorded seed:

* primitives by random-control rollouts, as the reference's
  ``generate_primitives_random`` does (src/motion_primitives/
  motion_primitives.cpp:498-577): canonical start, uniform controls per step,
  explicit-Euler rollout, then the loader's 1e-7 noise on the first and last
  state (src/ompl/robots.cpp:3113-3124) and, for the quadrotor, unit
  quaternions (src/ompl/robots.cpp:3127-3136);
* environments of random axis-aligned boxes;
* frontier states uniform over the free space.

The random stream is SplitMix64 in numpy integer arithmetic, so the same seed
gives the same inputs on every machine.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

UNICYCLE1, CAR1, QUAD3D, QUAD2D = 0, 1, 2, 3
ROBOT_NAMES = {UNICYCLE1: "unicycle1_v0", CAR1: "car1_v0", QUAD3D: "quadrotor_v0", QUAD2D: "quad2d_v0"}
NX = {UNICYCLE1: 3, CAR1: 4, QUAD3D: 13, QUAD2D: 6}
NU = {UNICYCLE1: 2, CAR1: 2, QUAD3D: 4, QUAD2D: 2}

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_C1 = np.uint64(0xBF58476D1CE4E5B9)
_C2 = np.uint64(0x94D049BB133111EB)


class Rng:
    """SplitMix64 stream (vectorised)."""

    def __init__(self, seed: int):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)

    def u64(self, n: int) -> np.ndarray:
        idx = np.arange(1, n + 1, dtype=np.uint64)
        with np.errstate(over="ignore"):
            s = self.state + idx * _GAMMA
            self.state = s[-1] if n > 0 else self.state
            z = s
            z = (z ^ (z >> np.uint64(30))) * _C1
            z = (z ^ (z >> np.uint64(27))) * _C2
            z = z ^ (z >> np.uint64(31))
        return z

    def uniform(self, n, lo=0.0, hi=1.0) -> np.ndarray:
        u = (self.u64(int(np.prod(n))) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return (lo + (hi - lo) * u).reshape(n)

    def integers(self, n, lo: int, hi: int) -> np.ndarray:
        """uniform integers in [lo, hi] (inclusive)"""
        span = np.uint64(hi - lo + 1)
        return (lo + (self.u64(n) % span).astype(np.int64)).astype(np.int64)

    def normal(self, n, sigma=1.0) -> np.ndarray:
        m = int(np.prod(n))
        u1 = self.uniform(m)
        u2 = self.uniform(m)
        z = np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * math.pi * u2)
        return (sigma * z).reshape(n)

    def unit_quaternions(self, n) -> np.ndarray:
        """uniform over SO(3), (x, y, z, w)"""
        u1, u2, u3 = self.uniform(n), self.uniform(n), self.uniform(n)
        a, b = np.sqrt(1 - u1), np.sqrt(u1)
        return np.stack([a * np.sin(2 * math.pi * u2), a * np.cos(2 * math.pi * u2),
                         b * np.sin(2 * math.pi * u3), b * np.cos(2 * math.pi * u3)], axis=-1)


# ------------------------------------------------------------------ robots --

@dataclasses.dataclass
class RobotModel:
    """Model constants; the field meaning is dpg_robot_desc's (include/dpg.h)."""
    kind: int
    nx: int
    nu: int
    n_parts: int
    dt: float
    w: tuple
    box: tuple = (0.0, 0.0)
    hitch: float = 0.0
    wheelbase: float = 0.0
    radius: float = 0.0
    mass: float = 0.0
    arm: float = 0.0
    t2t: float = 0.0
    inertia: tuple = (0.0, 0.0, 0.0)
    ang_gain: float = 0.0
    g: float = 9.81
    u_lb: tuple = ()
    u_ub: tuple = ()

    @property
    def name(self):
        return ROBOT_NAMES[self.kind]


def robot_model(kind: int) -> RobotModel:
    if kind == UNICYCLE1:
        return RobotModel(kind, 3, 2, 1, 0.1, (1.0, 0.5, 0.0, 0.0), box=(0.5, 0.25),
                          u_lb=(-0.5, -0.5), u_ub=(0.5, 0.5))
    if kind == CAR1:
        return RobotModel(kind, 4, 2, 2, 0.1, (1.0, 0.5, 0.5, 0.0), box=(0.5, 0.25), hitch=0.5,
                          wheelbase=0.25, u_lb=(-0.1, -math.pi / 3), u_ub=(0.5, math.pi / 3))
    if kind == QUAD3D:
        return RobotModel(kind, 13, 4, 1, 0.01, (1.0, 0.5, 0.1, 0.05), radius=0.1, mass=0.034,
                          arm=0.046, t2t=0.006, inertia=(16.571710e-6, 16.655602e-6, 29.261652e-6),
                          u_lb=(0.0,) * 4, u_ub=(1.4,) * 4)
    if kind == QUAD2D:
        return RobotModel(kind, 6, 2, 1, 0.01, (1.0, 0.5, 0.2, 0.1), box=(0.5, 0.25), ang_gain=34.0,
                          u_lb=(0.0, 0.0), u_ub=(1.4, 1.4))
    raise ValueError(kind)


def wrap_angle(x):
    """[-pi, pi): x - 2 pi floor((x + pi) / 2 pi), the planar models' angle
    normalisation"""
    return x - 2 * math.pi * np.floor((x + math.pi) / (2 * math.pi))


def step(m: RobotModel, x: np.ndarray, u: np.ndarray) -> np.ndarray:
    """Vectorised FP64 explicit-Euler step (rows of x and u)."""
    dt = m.dt
    xn = np.empty_like(x)
    if m.kind == UNICYCLE1:
        xn[:, 0] = x[:, 0] + u[:, 0] * np.cos(x[:, 2]) * dt
        xn[:, 1] = x[:, 1] + u[:, 0] * np.sin(x[:, 2]) * dt
        xn[:, 2] = wrap_angle(x[:, 2] + u[:, 1] * dt)
    elif m.kind == CAR1:
        xn[:, 0] = x[:, 0] + u[:, 0] * np.cos(x[:, 2]) * dt
        xn[:, 1] = x[:, 1] + u[:, 0] * np.sin(x[:, 2]) * dt
        xn[:, 2] = wrap_angle(x[:, 2] + u[:, 0] / m.wheelbase * np.tan(u[:, 1]) * dt)
        xn[:, 3] = wrap_angle(x[:, 3] + u[:, 0] / m.hitch * np.sin(x[:, 2] - x[:, 3]) * dt)
    elif m.kind == QUAD2D:
        acc = (u[:, 0] + u[:, 1]) * m.g * 0.5
        xn[:, 0] = x[:, 0] + x[:, 3] * dt
        xn[:, 1] = x[:, 1] + x[:, 4] * dt
        xn[:, 2] = wrap_angle(x[:, 2] + x[:, 5] * dt)
        xn[:, 3] = x[:, 3] - acc * np.sin(x[:, 2]) * dt
        xn[:, 4] = x[:, 4] + (acc * np.cos(x[:, 2]) - m.g) * dt
        xn[:, 5] = x[:, 5] + m.ang_gain * m.g * 0.5 * (u[:, 0] - u[:, 1]) * dt
    elif m.kind == QUAD3D:
        fu = m.mass * m.g * 0.25
        f = u * fu
        F = f.sum(1)
        lever = m.arm / math.sqrt(2.0)
        tau = np.stack([lever * (-f[:, 0] - f[:, 1] + f[:, 2] + f[:, 3]),
                        lever * (-f[:, 0] + f[:, 1] + f[:, 2] - f[:, 3]),
                        m.t2t * (-f[:, 0] + f[:, 1] - f[:, 2] + f[:, 3])], 1)
        q = x[:, 3:7]
        qx, qy, qz, qw = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
        am = F / m.mass
        acc = np.stack([2 * (qx * qz + qy * qw) * am, 2 * (qy * qz - qx * qw) * am,
                        (1 - 2 * (qx * qx + qy * qy)) * am - m.g], 1)
        J = np.array(m.inertia)
        w = x[:, 10:13]
        wd = (tau - np.cross(w, w * J)) / J
        hv = 0.5 * dt * w
        th = np.linalg.norm(hv, axis=1)
        sc = np.where(th > 1e-12, np.sin(th) / np.where(th > 1e-12, th, 1.0), 1.0)
        e = np.concatenate([hv * sc[:, None], np.cos(th)[:, None]], 1)
        ex, ey, ez, ew = e[:, 0], e[:, 1], e[:, 2], e[:, 3]
        qn = np.stack([qw * ex + qx * ew + qy * ez - qz * ey, qw * ey - qx * ez + qy * ew + qz * ex,
                       qw * ez + qx * ey - qy * ex + qz * ew, qw * ew - qx * ex - qy * ey - qz * ez], 1)
        qn /= np.linalg.norm(qn, axis=1, keepdims=True)
        xn[:, 0:3] = x[:, 0:3] + x[:, 7:10] * dt
        xn[:, 3:7] = qn
        xn[:, 7:10] = x[:, 7:10] + acc * dt
        xn[:, 10:13] = w + wd * dt
    return xn


# -------------------------------------------------------------- primitives --

@dataclasses.dataclass
class Primitives:
    """Motion set in the flattened layout dpg_upload_primitives takes."""
    length: np.ndarray   # int32 [P] states per motion
    states: np.ndarray   # float64 [sum L, nx]
    actions: np.ndarray  # float64 [sum (L-1), nu]

    @property
    def P(self):
        return len(self.length)

    def soff(self):
        return np.concatenate([[0], np.cumsum(self.length)[:-1]]).astype(np.int64)

    def aoff(self):
        return np.concatenate([[0], np.cumsum(self.length - 1)[:-1]]).astype(np.int64)

    def motion(self, p):
        s, a = self.soff()[p], self.aoff()[p]
        L = self.length[p]
        return self.states[s:s + L], self.actions[a:a + L - 1]


def canonical_starts(m: RobotModel, rng: Rng, P: int) -> np.ndarray:
    x0 = np.zeros((P, m.nx))
    if m.kind in (UNICYCLE1, QUAD2D):
        x0[:, 2] = rng.uniform(P, -math.pi, math.pi)
    if m.kind == CAR1:
        x0[:, 2] = rng.uniform(P, -math.pi, math.pi)
        x0[:, 3] = x0[:, 2] + rng.uniform(P, -math.pi / 4, math.pi / 4)
    if m.kind == QUAD2D:
        x0[:, 5] = rng.normal(P, 0.5)
    if m.kind == QUAD3D:
        x0[:, 3:7] = rng.unit_quaternions(P)
        x0[:, 10:13] = rng.normal((P, 3), 0.5)
    return x0


def make_primitives(m: RobotModel, P: int, steps_lo: int, steps_hi: int, seed: int,
                    noise: float = 1e-7) -> Primitives:
    """Random-control rollouts with canonical starts; steps uniform in
    [steps_lo, steps_hi] actions per primitive."""
    rng = Rng(seed)
    steps = rng.integers(P, steps_lo, steps_hi)
    x0 = canonical_starts(m, rng, P)
    T = int(steps.max())
    lb, ub = np.array(m.u_lb), np.array(m.u_ub)
    U = lb + (ub - lb) * rng.uniform((P, T, m.nu))
    X = np.empty((P, T + 1, m.nx))
    X[:, 0] = x0
    for k in range(T):
        X[:, k + 1] = step(m, X[:, k], U[:, k])
    length = (steps + 1).astype(np.int32)
    # loader noise on the first and last state (uniform in [-noise, noise])
    X[:, 0] += noise * rng.uniform((P, m.nx), -1.0, 1.0)
    last = X[np.arange(P), steps]
    X[np.arange(P), steps] = last + noise * rng.uniform((P, m.nx), -1.0, 1.0)
    if m.kind == QUAD3D:
        X[:, :, 3:7] /= np.linalg.norm(X[:, :, 3:7], axis=2, keepdims=True)
    states = np.concatenate([X[p, :length[p]] for p in range(P)], 0)
    actions = np.concatenate([U[p, :length[p] - 1] for p in range(P)], 0)
    return Primitives(length, np.ascontiguousarray(states), np.ascontiguousarray(actions))


def make_primitives_hover(m: RobotModel, P: int, steps_lo: int, steps_hi: int, seed: int, hold: int = 20,
                          tilt: float = 0.3, rate: float = 1.0, lift: tuple = (0.8, 1.25),
                          kp: float = 16.0, kd: float = 5.6, noise: float = 1e-7) -> Primitives:
    """quad2d motions that chain: canonical starts with |theta| <= tilt,
    |omega| <= rate and zero velocity; every `hold` steps a new tilt target in
    [-tilt, tilt] and lift factor in `lift` are drawn and a PD law on the
    angle (kp, kd in rad/s^2 per rad, per rad/s) sets the thrust difference,
    so the motion ends near level again.  The applied thrusts, clipped to
    the actuator bounds, are recorded as the motion's actions; then the
    loader's 1e-7 noise."""
    rng = Rng(seed)
    steps = rng.integers(P, steps_lo, steps_hi)
    x0 = np.zeros((P, m.nx))
    x0[:, 2] = rng.uniform(P, -tilt, tilt)
    x0[:, 5] = rng.uniform(P, -rate, rate)
    T = int(steps.max())
    n_hold = (T + hold - 1) // hold
    ref = rng.uniform((P, n_hold), -tilt, tilt)
    c = rng.uniform((P, n_hold), lift[0], lift[1])
    lb, ub = np.array(m.u_lb), np.array(m.u_ub)
    gain = m.ang_gain * m.g * 0.5
    X = np.empty((P, T + 1, m.nx))
    U = np.empty((P, T, m.nu))
    X[:, 0] = x0
    for k in range(T):
        j = k // hold
        th, om = X[:, k, 2], X[:, k, 5]
        d = (kp * (ref[:, j] - th) - kd * om) / gain
        base = c[:, j] / np.maximum(np.cos(th), 0.5)
        U[:, k] = np.clip(np.stack([base + 0.5 * d, base - 0.5 * d], 1), lb, ub)
        X[:, k + 1] = step(m, X[:, k], U[:, k])
    length = (steps + 1).astype(np.int32)
    X[:, 0] += noise * rng.uniform((P, m.nx), -1.0, 1.0)
    X[np.arange(P), steps] += noise * rng.uniform((P, m.nx), -1.0, 1.0)
    states = np.concatenate([X[p, :length[p]] for p in range(P)], 0)
    actions = np.concatenate([U[p, :length[p] - 1] for p in range(P)], 0)
    return Primitives(length, np.ascontiguousarray(states), np.ascontiguousarray(actions))


def make_search_problem(m: RobotModel, extent, n_obs_range, side, seed: int, margin: float = 0.05):
    """Environment with a random number of boxes in n_obs_range, and a start
    and a goal at rest (level, zero velocity) in free space."""
    rng = Rng(seed)
    n_obs = int(rng.integers(1, n_obs_range[0], n_obs_range[1])[0])
    env = make_env(extent, n_obs, side[0], side[1], seed + 1)
    out = []
    s = seed + 2
    while len(out) < 2:
        x = make_nodes(m, env, 8, seed=s, vel_sigma=0.0)
        s += 1
        x[:, 2:] = 0.0
        ok = state_gap(m, env, x) > margin
        out.extend(x[ok][: 2 - len(out)])
    return env, np.array(out[0]), np.array(out[1])


# ------------------------------------------------------------- environment --

@dataclasses.dataclass
class Env:
    lo: np.ndarray       # [dim] position bounds
    hi: np.ndarray
    obs_lo: np.ndarray   # [O, dim]
    obs_hi: np.ndarray

    @property
    def dim(self):
        return len(self.lo)


def make_env(extent, n_obs: int, side_lo: float, side_hi: float, seed: int) -> Env:
    rng = Rng(seed)
    ext = np.array(extent, dtype=np.float64)
    d = len(ext)
    c = rng.uniform((n_obs, d)) * ext
    side = rng.uniform((n_obs, d), side_lo, side_hi)
    return Env(np.zeros(d), ext, c - 0.5 * side, c + 0.5 * side)


def state_gap(m: RobotModel, env: Env, x: np.ndarray) -> np.ndarray:
    """min separating-axis gap of each state row against all obstacles"""
    oc = 0.5 * (env.obs_lo + env.obs_hi)
    oh = 0.5 * (env.obs_hi - env.obs_lo)
    if len(oc) == 0:
        return np.full(len(x), np.inf)
    if m.kind == QUAD3D:
        d = np.abs(x[:, None, 0:3] - oc[None]) - oh[None]
        mx = d.max(2)
        out = np.sqrt((np.maximum(d, 0) ** 2).sum(2))
        g = np.where(mx <= 0, mx, out) - m.radius
        return g.min(1)
    parts = [(x[:, 0], x[:, 1], x[:, 2])]
    if m.kind == CAR1:
        parts.append((x[:, 0] - m.hitch * np.cos(x[:, 3]), x[:, 1] - m.hitch * np.sin(x[:, 3]), x[:, 3]))
    a, b = 0.5 * m.box[0], 0.5 * m.box[1]
    best = np.full(len(x), np.inf)
    for cx, cy, th in parts:
        ct, st = np.cos(th)[:, None], np.sin(th)[:, None]
        ac, as_ = np.abs(ct), np.abs(st)
        dx, dy = cx[:, None] - oc[None, :, 0], cy[:, None] - oc[None, :, 1]
        gx = np.abs(dx) - (a * ac + b * as_ + oh[None, :, 0])
        gy = np.abs(dy) - (a * as_ + b * ac + oh[None, :, 1])
        gu = np.abs(dx * ct + dy * st) - (a + oh[None, :, 0] * ac + oh[None, :, 1] * as_)
        gv = np.abs(-dx * st + dy * ct) - (b + oh[None, :, 0] * as_ + oh[None, :, 1] * ac)
        g = np.maximum(np.maximum(gx, gy), np.maximum(gu, gv)).min(1)
        best = np.minimum(best, g)
    return best


def make_nodes(m: RobotModel, env: Env, N: int, seed: int, vel_sigma: float = 0.5,
               margin: float = 1e-3) -> np.ndarray:
    """N frontier states uniform over the free space (rejection sampling)."""
    rng = Rng(seed)
    out = []
    have = 0
    while have < N:
        k = max(1024, 2 * (N - have))
        x = np.zeros((k, m.nx))
        pd = 3 if m.kind == QUAD3D else 2
        x[:, :pd] = env.lo + (env.hi - env.lo) * rng.uniform((k, pd))
        if m.kind in (UNICYCLE1, QUAD2D):
            x[:, 2] = rng.uniform(k, -math.pi, math.pi)
        if m.kind == CAR1:
            x[:, 2] = rng.uniform(k, -math.pi, math.pi)
            x[:, 3] = x[:, 2] + rng.uniform(k, -math.pi / 4, math.pi / 4)
        if m.kind == QUAD2D:
            x[:, 3:5] = rng.normal((k, 2), vel_sigma)
            x[:, 5] = rng.normal(k, vel_sigma)
        if m.kind == QUAD3D:
            x[:, 3:7] = rng.unit_quaternions(k)
            x[:, 7:10] = rng.normal((k, 3), vel_sigma)
            x[:, 10:13] = rng.normal((k, 3), vel_sigma)
        ok = state_gap(m, env, x) > margin
        out.append(x[ok])
        have += int(ok.sum())
    return np.ascontiguousarray(np.concatenate(out, 0)[:N])


# ---------------------------------------------------------------- configs --

@dataclasses.dataclass
class Workload:
    name: str
    robot: RobotModel
    prims: Primitives
    env: Env
    nodes: np.ndarray
    delta: float
    alpha: float
    precision: int  # 0 FP32, 1 FP64
    seed: int

    @property
    def radius(self):
        return self.alpha * self.delta


# Sizes and parameters of the five workloads (the reference's db-A* default
# alpha = 0.5, include/dynoplan/dbastar/options.hpp:109-110).
CONFIGS = {
    1: dict(name="unicycle1_v0 plain FP64 expand", kind=UNICYCLE1, P=1000, steps=(5, 50),
            extent=(6.0, 6.0), n_obs=30, side=(0.2, 1.0), N=10_000, delta=0.3, precision=1),
    2: dict(name="car1_v0 batched FP32 expand", kind=CAR1, P=5000, steps=(5, 100),
            extent=(10.0, 10.0), n_obs=80, side=(0.2, 1.5), N=100_000, delta=0.3, precision=0),
    3: dict(name="quadrotor_v0 batched FP32 expand", kind=QUAD3D, P=5000, steps=(50, 300),
            extent=(6.0, 6.0, 3.0), n_obs=40, side=(0.2, 1.0), N=50_000, delta=0.8, precision=0),
    5: dict(name="quad2d_v0 end-to-end", kind=QUAD2D, P=10_000, steps=(20, 150),
            extent=(8.0, 4.0), n_obs=40, side=(0.2, 1.0), N=10_000, delta=0.5, precision=0,
            n_obs_range=(20, 60)),
}


def make_workload(cfg: int, scale: float = 1.0, seed: int | None = None, N: int | None = None,
                  P: int | None = None) -> Workload:
    """Workload `cfg`; `scale` shrinks P and N together for small test cases."""
    c = CONFIGS[cfg]
    seed = 1000 + cfg if seed is None else seed
    m = robot_model(c["kind"])
    P_ = P if P is not None else max(8, int(round(c["P"] * scale)))
    N_ = N if N is not None else max(8, int(round(c["N"] * scale)))
    prims = make_primitives(m, P_, c["steps"][0], c["steps"][1], seed)
    env = make_env(c["extent"], c["n_obs"], c["side"][0], c["side"][1], seed + 7)
    nodes = make_nodes(m, env, N_, seed + 13)
    return Workload(c["name"], m, prims, env, nodes, c["delta"], 0.5, c["precision"], seed)
