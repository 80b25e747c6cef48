"""CPU oracle of the learned closure (test infrastructure only).

Restates, in float64 numpy, what the CUDA kernels of cmag_gb300/csrc/closure.cu
compute: the 16 per-particle features (brute force over all pairs), the
16-64-64-64-3 SiLU network with BF16 parameters and BF16 activations, its loss
0.5/n sum |y - t|^2 and the gradient of that loss with respect to the
parameters (rounding treated as identity, as in the kernels).  BF16 rounding is
round-to-nearest-even on the float32 bit pattern.  The closure has no reference
counterpart, so this oracle is checked by finite differences
(tests/test_closure_oracle.py) rather than pinned to reference outputs.
"""
import numpy as np

FEAT, HIDDEN, OUT = 16, 64, 3
SHAPES = [("W1", (HIDDEN, FEAT)), ("b1", (HIDDEN,)), ("W2", (HIDDEN, HIDDEN)), ("b2", (HIDDEN,)),
          ("W3", (HIDDEN, HIDDEN)), ("b3", (HIDDEN,)), ("W4", (OUT, HIDDEN)), ("b4", (OUT,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def bf16(x):
    """Round float32 values to the nearest BF16 value (ties to even), as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(theta):
    out, k = {}, 0
    for name, shape in SHAPES:
        size = int(np.prod(shape))
        out[name] = np.asarray(theta[k:k + size], dtype=np.float64).reshape(shape)
        k += size
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def init_params(seed=0):
    """He-style initial parameters (what cmag_gb300.closure uses)."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in SHAPES:
        if name.startswith("W"):
            d[name] = rng.normal(0.0, np.sqrt(2.0 / shape[1]), size=shape)
        else:
            d[name] = np.zeros(shape)
    d["W4"] *= 0.1
    return pack(d).astype(np.float32)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(theta, feat, mean, inv_std, round_bf16=True):
    """Network outputs and the intermediate values the backward pass needs."""
    r = bf16 if round_bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    P = {k: r(v) for k, v in unpack(theta).items()}
    x = r((np.asarray(feat, np.float64) - mean) * inv_std)
    z1 = x @ P["W1"].T + P["b1"]
    a1 = r(silu(z1))
    z2 = a1 @ P["W2"].T + P["b2"]
    a2 = r(silu(z2))
    z3 = a2 @ P["W3"].T + P["b3"]
    a3 = r(silu(z3))
    y = a3 @ P["W4"].T + P["b4"]
    return y, (P, x, z1, a1, z2, a2, z3, a3)


def loss_and_grad(theta, feat, target, mean, inv_std, round_bf16=True):
    y, (P, x, z1, a1, z2, a2, z3, a3) = forward(theta, feat, mean, inv_std, round_bf16)
    n = y.shape[0]
    e = y - np.asarray(target, np.float64)
    loss = 0.5 * np.sum(e * e) / n
    dy = e / n
    g = {"W4": dy.T @ a3, "b4": dy.sum(0)}
    d3 = (dy @ P["W4"]) * dsilu(z3)
    g["W3"], g["b3"] = d3.T @ a2, d3.sum(0)
    d2 = (d3 @ P["W3"]) * dsilu(z2)
    g["W2"], g["b2"] = d2.T @ a1, d2.sum(0)
    d1 = (d2 @ P["W2"]) * dsilu(z1)
    g["W1"], g["b1"] = d1.T @ x, d1.sum(0)
    return loss, pack(g)


# ---------------------------------------------------------------- features ---

def wendland_w(q, w_norm):
    t = 1.0 - 0.5 * q
    return w_norm * t ** 4 * (2.0 * q + 1.0)


def wendland_dw(q, dw_norm):
    t = 1.0 - 0.5 * q
    return -2.5 * dw_norm * q * t ** 3


def features(p, pos, vel, rho, pres, acc, fluid_type=4):
    """Features of every fluid particle (rows of other particles are NaN).

    p: SphParams of a 3-D (dims 3) or 2-D Wendland DamBreak scene; pos, vel
    (leap-frog velocity), acc: (n, 4); rho, pres: (n,), all in one order."""
    pos = np.asarray(pos, np.float64)
    vel = np.asarray(vel, np.float64)
    h = float(np.float32(p.smoothing_radius))
    if int(p.dims) == 3:
        w_norm = 21.0 / (16.0 * np.pi * h ** 3)
    else:
        w_norm = 7.0 / (4.0 * np.pi * h ** 2)
    dw_norm = 2.0 * w_norm / h
    m, rho0, B, c0 = (float(np.float32(v)) for v in (p.particle_mass, p.rest_density, p.B, p.soundspeed))
    g = np.array([p.gravity[0], p.gravity[1], p.gravity[2]], np.float64)
    n = pos.shape[0]
    out = np.full((n, FEAT), np.nan)
    fluid = np.flatnonzero(pos[:, 3] == fluid_type)
    vol = m / np.asarray(rho, np.float64)
    wall = pos[:, 3] != fluid_type
    for i in fluid:
        r = pos[:, :3] - pos[i, :3]            # x_j - x_i
        d2 = np.sum(r * r, axis=1)
        nb = np.flatnonzero(d2 < 4.0 * h * h)
        d = np.sqrt(d2[nb])
        q = d / h
        vw = vol[nb] * wendland_w(q, w_norm)
        dv = vel[nb, :3] - vel[i, :3]
        f = out[i]
        f[0] = rho[i] / rho0 - 1.0
        f[1] = pres[i] / B
        f[2:5] = (vw[:, None] * r[nb]).sum(0) / h
        f[5:8] = (vw[:, None] * dv).sum(0) / c0
        f[8] = vw.sum()
        f[9] = (vw * d2[nb]).sum() / h ** 2
        f[10] = vw[wall[nb]].sum()
        f[11:14] = acc[i, :3] / np.linalg.norm(g)
        nz = d > 0
        gw = wendland_dw(q[nz], dw_norm) / d[nz]   # dW/dr / |r|
        dot = np.sum(dv[nz] * r[nb][nz], axis=1)
        f[14] = np.sum(-vol[nb][nz] * gw * dot) * h / c0
        f[15] = np.linalg.norm(vel[i, :3]) / c0
    return out
