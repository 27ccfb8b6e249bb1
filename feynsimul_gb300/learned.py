"""Learned bisection proposal: harvest, training and loading into the sampler.

No counterpart in the reference.  The plain sweep proposes each bisection midpoint from
the free-particle bridge N((x_l + x_r)/2, sigma_n^2) (FeynSimul/GPUsrc/kernel.c:306-362).
Here a small network (16-128-128-128-16, ReLU, BF16 weights, FP32 accumulation; kernels in
csrc/fs_mlp.cuh and csrc/fs_mlp_train.cu) predicts, for the level-1 midpoint of each
segment, a Gaussian N(mid + sigma_1 o, sigma_1^2 exp(s)) from the segment's endpoints.
The sweep draws from it and corrects the acceptance (Metropolis-Hastings), so the target
distribution is exact for any network; with zero output weights the proposal is the free
one.

Workflow::

    model = LearnedProposal(dof, sigma_1, length_scale)
    x, z = harvest_triples(paths, dof, N, S, sigma_1, length_scale)   # from plain-sampler paths
    model.train(x, z, steps=2000)                                     # GPU, own kernels
    kernel.setLearnedProposal(model)                                  # PIMCKernel(learnedProposal=True)

Features of a segment: (x_l + x_r)/2 and (x_r - x_l)/2 per degree of freedom times
1/length_scale, zero padded to 16.  Target: z = (x_mid - (x_l + x_r)/2) / sigma_1.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

IN, H, OUT = 16, 128, 16
SHAPES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
          ("W4", (OUT, H)), ("b4", (OUT,))]


def param_count():
    return sum(int(np.prod(s)) for _, s in SHAPES)


def unflatten(params):
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = params[o:o + n].reshape(shp)
        o += n
    return out


def to_bf16(x):
    """Round float32 values to BF16 (nearest even), returned as float32 values."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def bf16_bits(x):
    return (to_bf16(x).view(np.uint32) >> 16).astype(np.uint16)


def pack_fragments(params):
    """FP32 parameters -> (fragment-ordered BF16 weights as uint32 pairs, biases) in the
    layout fs_mlp_eval_warp reads (csrc/fs_mlp.cuh)."""
    p = unflatten(np.asarray(params, dtype=np.float32))
    blobs = []
    for name in ("W1", "W2", "W3", "W4"):
        W = p[name]                      # [N][K]
        N, K = W.shape
        kt, nt, lane = np.meshgrid(np.arange(K // 16), np.arange(N // 8), np.arange(32), indexing="ij")
        n = nt * 8 + lane // 4
        k = kt * 16 + (lane % 4) * 2
        lo0, hi0 = bf16_bits(W[n, k]), bf16_bits(W[n, k + 1])
        lo1, hi1 = bf16_bits(W[n, k + 8]), bf16_bits(W[n, k + 9])
        x = lo0.astype(np.uint32) | (hi0.astype(np.uint32) << 16)
        y = lo1.astype(np.uint32) | (hi1.astype(np.uint32) << 16)
        blobs.append(np.stack([x, y], axis=-1).reshape(-1, 2))   # order (kt, nt, lane)
    frag = np.ascontiguousarray(np.concatenate(blobs, axis=0))
    bias = np.ascontiguousarray(np.concatenate([p["b1"], p["b2"], p["b3"], p["b4"]]).astype(np.float32))
    return frag, bias


def init_params(seed=0, zero_output=True):
    """He-initialised hidden layers; the output layer starts at zero, i.e. the free proposal."""
    rng = np.random.RandomState(seed)
    chunks = []
    for name, shp in SHAPES:
        if name.startswith("b"):
            chunks.append(np.zeros(shp, np.float32))
        elif name == "W4" and zero_output:
            chunks.append(np.zeros(shp, np.float32))
        else:
            chunks.append((rng.randn(*shp) * np.sqrt(2.0 / shp[1])).astype(np.float32))
    return np.concatenate([c.ravel() for c in chunks]).astype(np.float32)


def features(x_left, x_right, length_scale):
    """(n, D) endpoints -> (n, 16) float32 features."""
    xl = np.asarray(x_left, dtype=np.float64)
    xr = np.asarray(x_right, dtype=np.float64)
    n, d = xl.shape
    f = np.zeros((n, IN), np.float32)
    f[:, :d] = 0.5 * (xl + xr) / length_scale
    f[:, d:2 * d] = 0.5 * (xr - xl) / length_scale
    return f


def harvest_triples(paths, dof, N, S, sigma1, length_scale, per_walker=None, rng=None):
    """Training data from equilibrium paths [walkers, DOF*N]: every segment start p gives the
    endpoints x[p], x[p + 2^S] and the level-1 midpoint x[p + 2^(S-1)] (periodic).  Returns
    (features [n, 16], targets z [n, 8])."""
    P = np.asarray(paths, dtype=np.float64).reshape(paths.shape[0], dof, N)
    seg = 2 ** S
    rng = rng or np.random.RandomState(0)
    W = P.shape[0]
    starts = np.arange(N) if per_walker is None else None
    if per_walker is None:
        w_idx = np.repeat(np.arange(W), N)
        p_idx = np.tile(starts, W)
    else:
        w_idx = np.repeat(np.arange(W), per_walker)
        p_idx = rng.randint(0, N, size=W * per_walker)
    xl = P[w_idx, :, p_idx]
    xm = P[w_idx, :, (p_idx + seg // 2) % N]
    xr = P[w_idx, :, (p_idx + seg) % N]
    feats = features(xl, xr, length_scale)
    z = np.zeros((xl.shape[0], 8), np.float32)
    z[:, :dof] = (xm - 0.5 * (xl + xr)) / sigma1
    return feats, z


def sigma_level(beta, N, S, n):
    """Free-particle bisection width at level n (kernel.c:608-618), in FP64."""
    return float(np.sqrt((2 ** S) * (beta / N) / (2.0 * 2 ** n)))


class LearnedProposal:
    """The network's parameters plus the constants that tie it to a system and a level."""

    def __init__(self, dof, sigma1, length_scale, params=None, seed=0):
        if not 1 <= dof <= 8:
            raise ValueError("the learned proposal supports 1 <= DOF <= 8")
        self.dof = dof
        self.sigma1 = float(sigma1)
        self.length_scale = float(length_scale)
        self.params = init_params(seed) if params is None else np.asarray(params, np.float32).copy()
        self.history = []

    # ---- packing for the sampler ----
    def packed(self):
        return pack_fragments(self.params)

    def save(self, filename):
        np.savez(filename, params=self.params, dof=self.dof, sigma1=self.sigma1,
                 length_scale=self.length_scale)

    @classmethod
    def load(cls, filename):
        z = np.load(filename)
        return cls(int(z["dof"]), float(z["sigma1"]), float(z["length_scale"]), params=z["params"])

    # ---- evaluation on the GPU with the sampler's device code ----
    def predict(self, feats):
        """Raw network outputs (n, 16) for features (n, 16), via fs_mlp_infer."""
        import torch
        L = _lib.lib()
        frag, bias = self.packed()
        dev = "cuda"
        tf = torch.from_numpy(frag.view(np.uint8).copy()).to(dev)
        tb = torch.from_numpy(bias).to(dev)
        tx = torch.from_numpy(np.ascontiguousarray(feats, np.float32)).to(dev)
        ty = torch.zeros((tx.shape[0], OUT), dtype=torch.float32, device=dev)
        s = torch.cuda.current_stream().cuda_stream
        _lib.check(L.fs_mlp_infer(tf.data_ptr(), tb.data_ptr(), tx.data_ptr(), ty.data_ptr(), tx.shape[0], s))
        torch.cuda.synchronize()
        return ty.cpu().numpy()

    def conditional(self, feats):
        """(mean shift o, std factor exp(s/2)) per DOF, in units of sigma_1."""
        y = self.predict(feats)
        o = y[:, :self.dof]
        s = 4.0 * np.tanh(0.25 * y[:, self.dof:2 * self.dof])
        return o, np.exp(0.5 * s)

    def validation_gain(self, feats, targets):
        """Held-out log-likelihood gain over the free-particle bridge, in nats per segment:
        the free proposal's negative log-likelihood (mean 0, width sigma_1) minus the
        network's, averaged over (feats, targets).  Positive means the network proposes the
        level-1 midpoint better than the plain bisection."""
        o, sd = self.conditional(feats)
        z = np.asarray(targets, np.float64)[:, :self.dof]
        nll = 0.5 * ((z - o) / sd) ** 2 + np.log(sd)
        return float(np.mean(np.sum(0.5 * z * z - nll, axis=1)))

    # ---- training on the GPU with the project's kernels ----
    def train(self, feats, targets, steps=2000, batch=4096, lr=1e-3, seed=0, log_every=0):
        """Adam on the Gaussian negative log-likelihood; returns the loss history (per step,
        mean over the batch)."""
        import torch
        L = _lib.lib()
        dev = "cuda"
        n = feats.shape[0]
        batch = min(batch, n)
        sizes = [ctypes.c_int64() for _ in range(4)]
        _lib.check(L.fs_mlp_sizes(*[ctypes.byref(v) for v in sizes]))
        n_param, n_bf16 = sizes[0].value, sizes[1].value
        assert n_param == self.params.size
        tp = torch.from_numpy(self.params.copy()).to(dev)
        tm = torch.zeros_like(tp)
        tv = torch.zeros_like(tp)
        tg = torch.zeros_like(tp)
        tq = torch.zeros(n_bf16, dtype=torch.int16, device=dev)
        frag_dummy = torch.zeros(sizes[2].value * 2, dtype=torch.int32, device=dev)
        bias_dummy = torch.zeros(sizes[3].value, dtype=torch.float32, device=dev)
        tx = torch.from_numpy(np.ascontiguousarray(feats, np.float32)).to(dev)
        tz = torch.from_numpy(np.ascontiguousarray(targets, np.float32)).to(dev)
        loss = torch.zeros(1, dtype=torch.float32, device=dev)
        stream = torch.cuda.current_stream().cuda_stream
        _lib.check(L.fs_mlp_pack(tp.data_ptr(), tq.data_ptr(), frag_dummy.data_ptr(), bias_dummy.data_ptr(), stream))
        gen = torch.Generator(device=dev)
        gen.manual_seed(seed)
        losses = torch.zeros(steps, dtype=torch.float32, device=dev)
        for it in range(steps):
            idx = torch.randint(0, n, (batch,), device=dev, generator=gen)
            xb = tx.index_select(0, idx).contiguous()
            zb = tz.index_select(0, idx).contiguous()
            loss.zero_()
            _lib.check(L.fs_mlp_train_step(tp.data_ptr(), tq.data_ptr(), tg.data_ptr(), xb.data_ptr(),
                                           zb.data_ptr(), batch, self.dof, 1.0 / batch, loss.data_ptr(), stream))
            _lib.check(L.fs_mlp_adam(tp.data_ptr(), tm.data_ptr(), tv.data_ptr(), tg.data_ptr(), tq.data_ptr(),
                                     it + 1, lr, stream))
            losses[it] = loss[0] / batch
            if log_every and (it + 1) % log_every == 0:
                print(f"step {it + 1}: loss {float(losses[it]):.4f}")
        torch.cuda.synchronize()
        self.params = tp.cpu().numpy().astype(np.float32)
        hist = losses.cpu().numpy()
        self.history.extend(hist.tolist())
        return hist


# ------------------------------------------------------------------ ESS study
def energy_series(kernel, launches, op_index=0):
    """Per-walker operator means of `launches` consecutive runs: (series[launch, walker],
    device seconds of the sweeps, wall seconds of the whole loop including the per-run
    reads of the operator means)."""
    import time
    series, t = [], 0.0
    t0 = time.perf_counter()
    for _ in range(launches):
        kernel.run()
        t += kernel.getRunTime()
        series.append(kernel.getOperators()[op_index])
    return np.array(series), t, time.perf_counter() - t0


def energy_ess(kernel, launches=200, burn=10):
    """Energy-estimator effective samples per second, the one definition this package
    reports: after ``burn`` runs, ``launches`` runs of the kernel (each run one operator
    measurement per walker, i.e. operatorRuns = 1), the integrated autocorrelation time of
    the per-walker energy series by Sokal's automatic window (stats.ess), and ESS divided by
    the wall time of the measured loop (sweeps, measurements and the reads of the
    per-walker energies)."""
    from .stats import ess, tau_int_batch_means
    for _ in range(burn):
        kernel.run()
    series, dev_s, wall_s = energy_series(kernel, launches)
    e, tau = ess(series)
    sweeps = kernel._operatorRuns * kernel._metroStepsPerOperatorRun
    return {"ess": float(e), "ess_per_s": float(e / wall_s), "tau_int_measurements": float(tau),
            "tau_int_sweeps": float(tau * sweeps), "tau_batch_means": float(tau_int_batch_means(series)),
            "measurements_per_walker": int(launches), "sweeps_per_measurement": int(sweeps),
            "wall_s": float(wall_s), "device_s": float(dev_s), "series": series}


def ess_study(system, beta, N, walkers, S_plain=(3, 4, 5, 6), S_learned=(4, 5, 6, 7), launches=200,
              op_runs=1, msteps=1, burn=10, train_steps=3000, harvest_snapshots=4, seed=1,
              kernel_extra=None, min_gain=0.01, force_network=(), log=print):
    """Energy-estimator ESS/s (energy_ess: per-sweep measurements by default, ESS over the
    wall time of the measured loop) of the plain sampler and of the learned proposal on one
    system.  Every sampler starts from the same equilibrated paths; a launch is op_runs x
    msteps sweeps followed by one operator measurement per walker and run.

    ``force_network``: levels S whose network is also measured when the gate rejects it
    (reported under ``results["forced"]``), so the network's own ESS/s is known.

    The learned sampler keeps the plain bisection as its fallback: a network whose held-out
    log-likelihood gain over the free bridge (LearnedProposal.validation_gain, on 10% of the
    harvested segments) is below ``min_gain`` nats per segment is not used, and that level
    runs the plain kernel (reported with ``fallback: True``)."""
    from .kernel import PIMCKernel
    from .kernel_args import KernelArgs
    extra = dict(kernel_extra or {})

    def make(S, learned, op_runs_=op_runs, msteps_=msteps):
        ka = KernelArgs(system=system, nbrOfWalkers=walkers, N=N, beta=float(beta), S=S, enableOperator=True,
                        enableCorrelator=False, enableBisection=True, enablePathShift=False,
                        enableSingleNodeMove=False, enableBins=False, nbrOfWalkersPerWorkGroup=1,
                        enableParallelizePath=True, enableGlobalPath=False, enableGlobalOldPath=False,
                        operators=(system.energyOp,), operatorRuns=op_runs_, metroStepsPerOperatorRun=msteps_,
                        seed=seed + 17 * S + (1000 if learned else 0), learnedProposal=learned, **extra)
        k = PIMCKernel(ka)
        if ka.enableRanlux:
            k.initRanlux()
            k.groupInitRanlux()
        return k

    rng = np.random.RandomState(seed)
    # equilibrate with the plain sampler at the middle level
    k0 = make(S_plain[len(S_plain) // 2], False, 5, 10)
    if hasattr(system, "initial_paths"):
        k0.setPaths(system.initial_paths(walkers, N, rng))
    for _ in range(burn):
        k0.run()
    snaps = []
    for _ in range(harvest_snapshots):
        k0.run()
        snaps.append(k0.getPaths())
    start_paths = snaps[-1].copy()
    k0.close()
    length_scale = float(np.sqrt(np.mean(np.concatenate(snaps) ** 2)))
    results = {"plain": {}, "learned": {}, "length_scale": length_scale}

    def measure(k, label):
        k.setPaths(start_paths)
        m = energy_ess(k, launches=launches, burn=3)
        series = m.pop("series")
        info = k.getInfo()
        nodes = walkers * (N // 2 ** k._S) * (2 ** k._S - 1) * op_runs * msteps * launches
        r = dict(m, S=k._S, node_updates_per_s=nodes / m["device_s"],
                 acceptance=float(k.getAcceptanceRate()), energy_mean=float(series.mean()),
                 energy_se=float(series.mean(axis=0).std() / np.sqrt(walkers)), registers=int(info.registers))
        log(f"{label} S={k._S}: AR {r['acceptance']:.3f} tau {r['tau_int_sweeps']:.2f} sweeps "
            f"ESS/s {r['ess_per_s']:.4g} nodes/s {r['node_updates_per_s']:.4g} E {r['energy_mean']:.5f}")
        return r

    for S in S_plain:
        k = make(S, False)
        results["plain"][S] = measure(k, "plain  ")
        k.close()
    for S in S_learned:
        s1 = sigma_level(beta, N, S, 1)
        feats, z = [], []
        for P in snaps:
            f, t = harvest_triples(P, system.DOF, N, S, s1, length_scale, per_walker=64, rng=rng)
            feats.append(f)
            z.append(t)
        feats, z = np.concatenate(feats), np.concatenate(z)
        n_val = max(1, feats.shape[0] // 10)
        model = LearnedProposal(system.DOF, s1, length_scale, seed=seed)
        hist = model.train(feats[n_val:], z[n_val:], steps=train_steps, batch=8192, lr=1e-3, seed=seed)
        gain = model.validation_gain(feats[:n_val], z[:n_val])
        info = dict(train_samples=int(feats.shape[0] - n_val), loss_start=float(hist[:20].mean()),
                    loss_end=float(hist[-50:].mean()), validation_gain_nats=gain)
        if gain < min_gain and S in force_network:
            k = make(S, True)
            k.setLearnedProposal(model)
            results.setdefault("forced", {})[S] = dict(measure(k, "forced "), fallback=False, **info)
            k.close()
        if gain < min_gain:
            if S not in results["plain"]:
                k = make(S, False)
                results["plain"][S] = measure(k, "plain  ")
                k.close()
            r = dict(results["plain"][S], fallback=True, **info)
            log(f"learned S={S}: validation gain {gain:.4f} nats < {min_gain}: plain bisection (fallback)")
        else:
            k = make(S, True)
            k.setLearnedProposal(model)
            r = measure(k, "learned")
            r.update(fallback=False, **info)
            k.close()
        results["learned"][S] = r
    best_plain = max(results["plain"].values(), key=lambda r: r["ess_per_s"])
    best_learned = max(results["learned"].values(), key=lambda r: r["ess_per_s"])
    used = [r for r in results["learned"].values() if not r["fallback"]]
    best_net = max(used, key=lambda r: r["ess_per_s"]) if used else None
    ref = results["plain"].get(4, best_plain)
    # Any proposal, learned or not: one measurement per sweep, ESS = measurements / (2 tau_int)
    # with Sokal's tau_int >= 1/2, and a sweep no cheaper than the plain one at its S, so its
    # ESS/s is at most the fastest plain measurement rate (ESS/s x 2 tau_int).
    rate_max = max(r["ess_per_s"] * 2.0 * r["tau_int_measurements"] for r in results["plain"].values())
    results["summary"] = {
        "plain_S4_ess_per_s": ref["ess_per_s"], "best_plain_S": best_plain["S"],
        "best_plain_ess_per_s": best_plain["ess_per_s"], "best_learned_S": best_learned["S"],
        "best_learned_ess_per_s": best_learned["ess_per_s"],
        "best_learned_is_fallback": bool(best_learned["fallback"]),
        "learned_vs_plain_S4": best_learned["ess_per_s"] / ref["ess_per_s"],
        "learned_vs_best_plain": best_learned["ess_per_s"] / best_plain["ess_per_s"],
        "network_levels_used": sorted(int(r["S"]) for r in used),
        "network_only_vs_best_plain": (best_net["ess_per_s"] / best_plain["ess_per_s"]) if best_net else None,
        "network_forced": {int(S): {"ess_per_s": r["ess_per_s"], "acceptance": r["acceptance"],
                                    "tau_int_sweeps": r["tau_int_sweeps"],
                                    "vs_plain_same_S": r["ess_per_s"] / results["plain"][S]["ess_per_s"]
                                    if S in results["plain"] else None}
                           for S, r in results.get("forced", {}).items()},
        "validation_gain_nats": {int(S): r["validation_gain_nats"] for S, r in results["learned"].items()},
        "any_proposal_bound_vs_best_plain": rate_max / best_plain["ess_per_s"]}
    return results
