"""The learned closure: binding, training data and training loop.

A coarse DamBreak run (twice the particle spacing of a fine one, an eighth of the
particles) misses the sub-grid part of the pressure, viscous and wall
accelerations.  The closure -- a 16-64-64-64-3 SiLU network with BF16 parameters
and activations, evaluated by the library's own CUDA kernels after the force
stage -- predicts that part per fluid particle.

Training data come from the solver itself: a fine run and a coarse run of the
same seeded scene advance in lockstep with the plain method (the coarse run
starts from the 2x2x2 block means of the fine initial state: the coarse lattice
plus the fine jitter averaged over each block).  At each sampled instant the
library extracts the coarse state's features, and the target of every coarse
fluid particle is the fine run's acceleration field at that particle's position
(Shepard-normalised SPH interpolation over the fine fluid, cmag_system_interpolate)
minus the coarse run's own plain acceleration; particles outside the fine fluid
(Shepard sum below a threshold) are left out.  The samples are thus states the
coarse method itself visits.  Device memory for the data comes from torch
(plumbing only; every computation is a library kernel).
"""
import ctypes

import numpy as np

from . import _abi
from ._lib import c_f32p, check, lib

NFEAT, NOUT = 16, 3


def _fp(a):
    return a.ctypes.data_as(c_f32p)


def _ptr(t):
    return ctypes.c_void_p(int(t.data_ptr()) if hasattr(t, "data_ptr") else int(t))


class Closure:
    def __init__(self, params=None):
        self.nparams = int(lib().cmag_closure_param_count())
        self._h = ctypes.c_void_p()
        arr = None
        if params is not None:
            arr = np.ascontiguousarray(params, dtype=np.float32)
            if arr.size != self.nparams:
                raise ValueError("expected %d parameters" % self.nparams)
        check(lib().cmag_closure_create(_fp(arr) if arr is not None else None, ctypes.byref(self._h)))

    def close(self):
        if getattr(self, "_h", None):
            lib().cmag_closure_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        return check(rc, closure=self._h)

    @property
    def params(self):
        out = np.empty(self.nparams, np.float32)
        self._chk(lib().cmag_closure_get_params(self._h, _fp(out)))
        return out

    @params.setter
    def params(self, v):
        a = np.ascontiguousarray(v, dtype=np.float32)
        self._chk(lib().cmag_closure_set_params(self._h, _fp(a)))

    def bf16_params(self):
        out = np.empty(self.nparams, np.float32)
        self._chk(lib().cmag_closure_get_bf16_params(self._h, _fp(out)))
        return out

    def set_normalization(self, mean, inv_std, out_scale):
        m = np.ascontiguousarray(mean, dtype=np.float32)
        s = np.ascontiguousarray(inv_std, dtype=np.float32)
        self._chk(lib().cmag_closure_set_normalization(self._h, _fp(m), _fp(s), float(out_scale)))

    def set_output_limit(self, limit):
        self._chk(lib().cmag_closure_set_output_limit(self._h, float(limit)))

    def normalization(self):
        m = np.empty(NFEAT, np.float32)
        s = np.empty(NFEAT, np.float32)
        o = np.empty(1, np.float32)
        self._chk(lib().cmag_closure_get_normalization(self._h, _fp(m), _fp(s), _fp(o)))
        return m, s, float(o[0])

    def forward(self, feat, out, n=None, stream=None):
        n = feat.shape[0] if n is None else int(n)
        self._chk(lib().cmag_closure_forward(self._h, _ptr(feat), n, _ptr(out), stream))

    def gradient(self, feat, target, n=None, stream=None):
        n = feat.shape[0] if n is None else int(n)
        g = np.empty(self.nparams, np.float32)
        loss = np.empty(1, np.float32)
        self._chk(lib().cmag_closure_gradient(self._h, _ptr(feat), _ptr(target), n, _fp(g), _fp(loss), stream))
        return float(loss[0]), g

    def train_step(self, feat, target, lr, n=None, want_loss=False, stream=None):
        n = feat.shape[0] if n is None else int(n)
        loss = np.empty(1, np.float32)
        self._chk(lib().cmag_closure_train_step(self._h, _ptr(feat), _ptr(target), n, float(lr),
                                                _fp(loss) if want_loss else None, stream))
        return float(loss[0]) if want_loss else None

    def reset_optimizer(self):
        self._chk(lib().cmag_closure_reset_optimizer(self._h))

    def synchronize(self):
        self._chk(lib().cmag_closure_synchronize(self._h))


# ------------------------------------------------------------ training data ---

def block_index(fluid):
    """(coarse fluid count, 8) original indices of the fine fluid particles of each
    2x2x2 lattice block (fluid rows come first, x fastest), blocks in the coarse
    lattice's order."""
    fx, fy, fz = fluid
    z, y, x = np.meshgrid(np.arange(0, fz, 2), np.arange(0, fy, 2), np.arange(0, fx, 2), indexing="ij")
    base = (x + fx * (y + fy * z)).ravel()
    corners = [dx + fx * (dy + fy * dz) for dz in (0, 1) for dy in (0, 1) for dx in (0, 1)]
    return base[:, None] + np.array(corners)[None, :]


class Pair:
    """A fine and a coarse 3-D dam break of the same tank (coarse spacing 2x)."""

    def __init__(self, fluid=(64, 128, 64), tank=(256, 192, 64), layers=3, dt_fine=5e-5, alpha=0.01):
        from . import presets
        from .systems import DamBreakSystem
        self.fluid_f = tuple(fluid)
        self.fluid_c = tuple(v // 2 for v in fluid)
        self.tank_f, self.tank_c, self.layers = tuple(tank), tuple(v // 2 for v in tank), layers
        self.pf, self.nf, _, _ = presets.dambreak3d(fluid=self.fluid_f, tank=self.tank_f, layers=layers,
                                                     dt=dt_fine, alpha=alpha)
        self.pc, self.nc, _, _ = presets.dambreak3d(fluid=self.fluid_c, tank=self.tank_c, layers=layers,
                                                     dt=2 * dt_fine, alpha=alpha)
        self.fine = DamBreakSystem(params=self.pf, num_particles=self.nf)
        self.coarse = DamBreakSystem(params=self.pc, num_particles=self.nc)
        self.nfluid_c = int(np.prod(self.fluid_c))
        self.blocks = block_index(self.fluid_f)
        # the coarse scene's own walls (its fluid rows are replaced by block means)
        self.coarse.scene3d(self.tank_c, layers, 0.0, 0)
        self.coarse_walls = self.coarse.getArray(_abi.POSITION)[self.nfluid_c:]

    def start(self, seed):
        """Fine scene with jitter seed `seed` at t = 0, and the coarse run's
        initial state from its block means."""
        self.fine.scene3d(self.tank_f, self.layers, 0.01, seed)
        self.coarse_state_from_fine()

    def block_mean(self, array):
        """Per coarse fluid particle, the mean of `array` (original order) over
        its fine block."""
        a = self.fine.getArray(array)
        return a[self.blocks].mean(axis=1, dtype=np.float64).astype(np.float32)

    def coarse_state_from_fine(self, system=None):
        """Load the block means of the fine state (+ coarse walls) into `system`
        (default: the coarse solver)."""
        s = self.coarse if system is None else system
        pos = self.block_mean(_abi.POSITION)
        pos[:, 3] = _abi.FLUID
        out = {_abi.POSITION: np.concatenate([pos, self.coarse_walls])}
        for a in (_abi.VELOCITY, _abi.VELOCITYLEAPFROG):
            v = np.zeros((self.nc, 4), np.float32)
            v[:self.nfluid_c] = self.block_mean(a)
            out[a] = v
        meas = np.zeros((self.nc, 4), np.float32)
        meas[:, 0] = self.pc.rest_density
        out[_abi.MEASURES] = meas
        out[_abi.ACCELERATION] = np.zeros((self.nc, 4), np.float32)
        for a, v in out.items():
            s.setArray(a, v)
        s.set_elapsed_time(self.fine.getElapsedTime())

    def sample(self, feat_dev, target_dev, row0, min_shepard=0.5):
        """Features and targets of the current (fine, coarse) pair of states into
        rows row0.. of the device arrays; returns the number of rows written."""
        import torch
        self.coarse.set_closure(None)
        self.fine.run_stages(_abi.STAGE_FORCE)
        self.coarse.run_stages(_abi.STAGE_FORCE)
        n = self.nfluid_c
        full = torch.empty((self.nc, NFEAT), dtype=torch.float32, device="cuda")
        self.coarse.closure_features(full.data_ptr())
        a_coarse = torch.from_numpy(self.coarse.getArray(_abi.ACCELERATION)[:n, :3].copy()).cuda()
        pts = torch.from_numpy(self.coarse.getArray(_abi.POSITION)[:n].copy()).cuda()
        interp = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        self.fine.interpolate(_abi.ACCELERATION, pts.data_ptr(), n, interp.data_ptr())
        keep = interp[:, 3] >= min_shepard
        k = int(keep.sum())
        feat_dev[row0:row0 + k] = full[:n][keep]
        target_dev[row0:row0 + k] = (interp[:, :3] - a_coarse)[keep]
        return k

    def missed(self, min_shepard=0.5):
        """The coarse run's missed acceleration at the current pair of states: the
        fine acceleration field at each coarse fluid particle minus the coarse
        run's own (device (n, 3)), and whether the fine fluid reaches the particle
        (device bool (n,))."""
        import torch
        self.coarse.set_closure(None)
        self.fine.run_stages(_abi.STAGE_FORCE)
        self.coarse.run_stages(_abi.STAGE_FORCE)
        n = self.nfluid_c
        a_coarse = torch.from_numpy(self.coarse.getArray(_abi.ACCELERATION)[:n, :3].copy()).cuda()
        pts = torch.from_numpy(self.coarse.getArray(_abi.POSITION)[:n].copy()).cuda()
        interp = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        self.fine.interpolate(_abi.ACCELERATION, pts.data_ptr(), n, interp.data_ptr())
        return interp[:, :3] - a_coarse, interp[:, 3] >= min_shepard

    def features(self):
        """The coarse run's closure features at its current state (device (n, 16))."""
        import torch
        self.coarse.set_closure(None)
        self.coarse.run_stages(_abi.STAGE_FORCE)
        full = torch.empty((self.nc, NFEAT), dtype=torch.float32, device="cuda")
        self.coarse.closure_features(full.data_ptr())
        return full[:self.nfluid_c]

    def close(self):
        self.fine.close()
        self.coarse.close()


def normalization_from(feat_dev, target_dev, chunk=1 << 24):
    """Feature mean / inverse std and the target scale over a dataset (sums in
    FP64, a chunk of rows at a time, so the data set is never copied whole)."""
    import torch
    n = feat_dev.shape[0]
    s1 = torch.zeros(feat_dev.shape[1], dtype=torch.float64, device=feat_dev.device)
    s2 = torch.zeros_like(s1)
    t2 = torch.zeros((), dtype=torch.float64, device=feat_dev.device)
    for a in range(0, n, chunk):
        f = feat_dev[a:a + chunk].double()
        s1 += f.sum(0)
        s2 += f.pow(2).sum(0)
        t2 += target_dev[a:a + chunk].double().pow(2).sum()
    mean = s1 / n
    # unbiased variance, as torch.std
    var = ((s2 - n * mean * mean) / max(n - 1, 1)).clamp_min(0.0)
    std = var.sqrt().clamp_min(1e-6)
    scale = float((t2 / (n * target_dev.shape[1])).sqrt().clamp_min(1e-9))
    return mean.float().cpu().numpy(), (1.0 / std).float().cpu().numpy(), scale


def output_limit_from(target_dev, scale, q=0.999):
    """Twice the q-quantile of the scaled target magnitudes: the clamp that keeps
    a coarse run's corrections within what the training data showed."""
    import torch
    m = (target_dev.abs() / scale).flatten()
    if m.numel() > 1 << 23:
        m = m[torch.randint(0, m.numel(), (1 << 23,), device=m.device)]
    return 2.0 * float(torch.quantile(m.float(), q))


def train(closure, feat_dev, target_dev, steps, batch=65536, lr=2e-3, lr_final=2e-4, seed=0,
          log_every=0):
    """Adam over random minibatches of the (features, targets / out_scale) rows."""
    import torch
    _, _, scale = closure.normalization()
    tgt = (target_dev / scale).contiguous()
    n = feat_dev.shape[0]
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    # the library's kernels run on torch's stream, ordered with the gathers
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    losses = []
    for k in range(steps):
        rows = torch.randint(0, n, (min(batch, n),), device="cuda", generator=g)
        f = feat_dev[rows].contiguous()
        t = tgt[rows].contiguous()
        lr_k = lr * (lr_final / lr) ** (k / max(steps - 1, 1))
        want = log_every and (k % log_every == 0 or k == steps - 1)
        loss = closure.train_step(f, t, lr_k, want_loss=bool(want), stream=stream)
        if want:
            losses.append((k, loss))
    torch.cuda.current_stream().synchronize()
    return losses


# ------------------------------------------------------------------ rollouts ---

def front(system, column_width):
    """Surge front over the initial column width: the largest x of a fluid
    particle (DamBreak.Report/XFrontTest.h:64,79-86, reduced on the device) plus
    the particle radius, i.e. the free surface, so that runs at different spacings
    compare (at t = 0 both give the column's face)."""
    _, hi = system.fluid_extent()
    return (hi[0] + float(system.params.particle_radius)) / column_width


def rollout(system, t_end, sample_dt, column_width, steps_per_call=None):
    """Advance `system` to t_end; returns (device seconds spent stepping, sample
    times, fronts).  Fronts are read between timed calls, outside the timing."""
    dt = float(system.params.delta_time)
    per = max(1, int(round(sample_dt / dt)))
    total = int(round(t_end / dt))
    ms = 0.0
    times, fronts = [0.0], [front(system, column_width)]
    done = 0
    while done < total:
        k = min(per, total - done)
        ms += system.timed_update(k)
        done += k
        times.append(done * dt)
        fronts.append(front(system, column_width))
    system.synchronize()
    return ms / 1e3, np.array(times), np.array(fronts)


def collect(pair, seeds, snapshots, every, min_shepard=0.5):
    """Training rows from lockstep fine/coarse runs of the given jitter seeds:
    `snapshots` samples per seed, `every` fine steps (every / 2 coarse steps)
    apart.  Returns device (features, targets)."""
    import torch
    if every % 2:
        raise ValueError("the coarse run takes one step per two fine steps: `every` must be even")
    rows = len(seeds) * snapshots * pair.nfluid_c
    feat_dev = torch.empty((rows, NFEAT), dtype=torch.float32, device="cuda")
    target_dev = torch.empty((rows, NOUT), dtype=torch.float32, device="cuda")
    row = 0
    for seed in seeds:
        pair.start(seed)
        for _ in range(snapshots):
            pair.fine.update_n(every)
            pair.coarse.update_n(every // 2)
            row += pair.sample(feat_dev, target_dev, row, min_shepard)
    return feat_dev[:row].contiguous(), target_dev[:row].contiguous()


def collect_filtered(pair, seeds, snapshots, every, window, min_shepard=0.5, deadline=None, done=None):
    """Training rows with time-filtered targets: along the lockstep fine/coarse
    runs of each seed (no restarts), the target of a coarse fluid particle is its
    missed acceleration averaged over the `window` coarse steps that end at the
    sample (the acoustic part, which the two resolutions do not share, averages
    out; what the coarse method misses systematically stays), and its features
    are those at the sample.  `every` fine steps between samples (even, at least
    2 window).  With a `deadline` (time.perf_counter() value) no seed starts after
    it; `done` (a list) receives the seeds collected.  Returns device (features,
    targets)."""
    import time
    import torch
    if every % 2 or every < 2 * window:
        raise ValueError("`every` must be even and at least 2 * window")
    n = pair.nfluid_c
    rows = len(seeds) * snapshots * n
    feat_dev = torch.empty((rows, NFEAT), dtype=torch.float32, device="cuda")
    target_dev = torch.empty((rows, NOUT), dtype=torch.float32, device="cuda")
    row = 0
    for seed in seeds:
        if deadline is not None and time.perf_counter() > deadline:
            break
        if done is not None:
            done.append(seed)
        pair.start(seed)
        for _ in range(snapshots):
            lead = every - 2 * window
            pair.fine.update_n(lead)
            pair.coarse.update_n(lead // 2)
            acc = torch.zeros((n, NOUT), dtype=torch.float32, device="cuda")
            cnt = torch.zeros(n, dtype=torch.float32, device="cuda")
            for _w in range(window):
                pair.fine.update_n(2)
                pair.coarse.update_n(1)
                t, keep = pair.missed(min_shepard)
                kf = keep.float()
                acc += t * kf[:, None]
                cnt += kf
            keep = cnt >= 0.5 * window
            k = int(keep.sum())
            feat_dev[row:row + k] = pair.features()[keep]
            target_dev[row:row + k] = (acc / cnt.clamp_min(1.0)[:, None])[keep]
            row += k
    return feat_dev[:row].contiguous(), target_dev[:row].contiguous()


def front_errors(fronts, fine_fronts, tank_over_column):
    """Max and mean relative front error against the fine run while the fine
    front is short of the far wall."""
    judged = fine_fronts < 0.95 * tank_over_column
    err = np.abs(fronts - fine_fronts) / fine_fronts
    return float(err[judged].max()), float(err[judged].mean())


def choose_strength(pair, closure, seed, t_end, column_width, factors=(0.0, 0.25, 0.5, 0.75, 1.0),
                    sample_dt=0.01):
    """The fine run judges the closure: on a validation seed (not a training or
    held-out seed), roll the coarse run out with the correction scaled by each
    factor (0 = the plain coarse method) and keep the factor whose surge front
    stays closest to the fine run's (smallest maximum relative error).  Sets the
    closure's output scale accordingly and returns (factor, {factor: (max, mean)})."""
    mean, inv, scale = closure.normalization()
    tank_over_column = pair.tank_f[0] / pair.fluid_f[0]
    pair.start(seed)
    _, _, fine = rollout(pair.fine, t_end, sample_dt, column_width)
    errs = {}
    for f in factors:
        pair.start(seed)
        if f > 0.0:
            closure.set_normalization(mean, inv, scale * f)
            pair.coarse.set_closure(closure)
        else:
            pair.coarse.set_closure(None)
        _, _, fr = rollout(pair.coarse, t_end, sample_dt, column_width)
        errs[f] = front_errors(fr, fine, tank_over_column)
    pair.coarse.set_closure(None)
    best = min(factors, key=lambda f: (errs[f][0], errs[f][1]))
    closure.set_normalization(mean, inv, scale * max(best, 0.0))
    return best, errs
