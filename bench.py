"""Benchmark: term-gate applications per second of truncated Pauli propagation on
the 100-qubit 10x10 kicked-Ising circuit (20 Trotter steps; RZZ(-pi/2) on the
180 lattice edges then RX(theta_h) on every site; observable Z at site (5,5);
maximum weight 8, coefficient threshold 1e-6), swept over
theta_h in {0.1, 0.3, 0.5, 0.7, 0.9, 1.1, pi/2}.

One step = the whole theta_h sweep: by default its 7 values run as instances
of one batched propagation with per-instance angles (each instance's terms
bit-identical to its own propagation); --sweep separate runs 7 propagations.
Term-gate applications ("apps") = sum over rotation gates of the live terms
entering the gate.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload kicked_ising|kicked_ising_w10|hubbard|hea]

--workload hubbard measures the 6x6 Fermi-Hubbard Majorana propagation (144
Majoranas, 10 Trotter steps, degree <= 6, tau = 1e-7) instead; one step = one
propagation.  --workload hea measures 256 instances of a 50-qubit ansatz in one
batched propagation plus the adjoint gradient of every angle.  --workload
kicked_ising_w10 runs the kicked-Ising circuit at maximum weight 10 (theta_h =
0.3), the large-N case with ~4e8 terms inside a batch at the peak.

Prints one JSON line on rank 0.  Multi-GPU runs are independent replicas (the
propagation of one observable does not shard without a per-gate exchange):
every rank runs the full sweep on its own GPU, value = total apps / max time.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

UNIT = "apps/s"
MAXDEG, TAU = 8, 1e-6
OBS_SITE = 55


class KickedIsing:
    """10x10 kicked Ising (the headline workload); one step = the theta_h sweep."""
    name = "kicked_ising_10x10_w8_tau1e-6"
    metric = "term-gate applications/s (10x10 kicked Ising, 20 steps, W=8, tau=1e-6, theta_h sweep)"
    kind = "pauli"
    bytes_per_term = 32 + 8  # 128-bit x and z masks + FP64 coefficient (real mode)
    kernel = "orbit engine (orbit_classify..orbit_process_big) + persistent per-gate kernel"
    launch_unit = "one commuting run (orbit batch) or one persistent run"
    # DRAM bytes per orbit batch from one ncu capture (dram__bytes_read.sum +
    # dram__bytes_write.sum over every kernel of one theta_h = 0.5 propagation:
    # 43.5 MB read, 0 B written, 40 batches); the term store stays in L2.
    # DRAM bytes of one propagation from one ncu capture (dram__bytes_read.sum +
    # dram__bytes_write.sum over every kernel of the theta_h = 0.5 propagation:
    # 43.5 MB read, 0 B written); the term store stays in L2.
    dram_per_propagation = 43.5e6

    @property
    def traffic(self):
        """DRAM bytes per step (one propagation per theta_h), scaled from the
        theta_h = 0.5 capture."""
        return self.dram_per_propagation * len(self.thetas)

    traffic_note = ("per step: ncu dram__bytes_read.sum + dram__bytes_write.sum of all kernels of one "
                    "theta_h=0.5 propagation (43.5 MB read, 0 written) x the propagations of a step")
    # the same counters over every kernel of one step of the batched sweep (317
    # launches: 146.3 MB read, 0 written)
    dram_per_batched_step = 146.3e6
    batched_traffic_note = ("per step: ncu dram__bytes_read.sum + dram__bytes_write.sum over all 317 kernels "
                            "of one batched-sweep step (146.3 MB read, 0 written)")
    thetas = (0.1, 0.3, 0.5, 0.7, 0.9, 1.1, math.pi / 2)
    maxdeg = MAXDEG
    cpu_steps = 20  # Trotter steps of each propagation in the CPU sample
    serial_steps = 20  # Trotter steps of each propagation in the one-core sample

    @property
    def params(self):
        return dict(maxdegree=self.maxdeg, topk=0, mincoeff=TAU, max_xweight=-1, xtrunc_period=1,
                    batched=1, deterministic=0)

    def tables(self, steps=20):
        import fastfermion_gb300 as ff
        return [ff.encode_pauli_circuit(ff.build_circuit(ff.workloads.kicked_ising_circuit(th, steps=steps)))
                for th in self.thetas]

    def observable(self):
        keys = np.zeros((4, 1), dtype=np.uint64)
        keys[2, 0] = np.uint64(1) << np.uint64(OBS_SITE)
        return keys, np.ones(1), np.zeros(1)

    def propagate(self, ctx, k, re, im, tab, n=None):
        p = dict(self.params)
        if n is not None:
            p["n"] = n
        return ctx.pauli_propagate(k, re, im, tab, p, on_device=n is not None)

    def cpu_sample(self, tabs, cores, min_seconds=0.0):
        """The oracle's sharded OpenMP port of the reference on the whole theta_h
        sweep, repeated until min_seconds of CPU time have passed."""
        from oracle import oracle as O
        keys, re, im = self.observable()
        if self.cpu_steps != 20:
            tabs = self.tables(self.cpu_steps)
        apps, sweeps = 0, 0
        t0 = time.perf_counter()
        while sweeps == 0 or time.perf_counter() - t0 < min_seconds:
            for tab in tabs:
                apps += O.pauli_propagate(tab, keys, re, im, maxdegree=self.maxdeg, mincoeff=TAU,
                                          n_threads=cores).apps
            sweeps += 1
        part = "" if self.cpu_steps == 20 else f" (first {self.cpu_steps} of 20 Trotter steps)"
        return apps, time.perf_counter() - t0, cores, (
            f"{sweeps} x the theta_h sweep of the same workload{part}, sharded OpenMP port "
            "of the reference algorithm")

    def ref_sample(self, ref, cores, apps_cache):
        """The reference itself (its sharded OpenMP strategy, `cores` threads) on
        the whole theta_h sweep (first cpu_steps Trotter steps); the apps of each
        propagation are the oracle's count, computed once (apps_cache)."""
        import fastfermion_gb300 as ff
        obs = ref.poly(f"Z{OBS_SITE}")
        if "circs" not in apps_cache:
            from oracle import oracle as O
            keys, re, im = self.observable()
            apps_cache["circs"], apps_cache["apps"] = [], []
            for th in self.thetas:
                spec = ff.workloads.kicked_ising_circuit(th, steps=self.cpu_steps)
                apps_cache["circs"].append([ref.ROT(g[1], list(g[2]), g[3]) for g in spec])
                tab = ff.encode_pauli_circuit(ff.build_circuit(spec))
                apps_cache["apps"].append(O.pauli_propagate(tab, keys, re, im, maxdegree=self.maxdeg, mincoeff=TAU,
                                                            n_threads=cores).apps)
        t0 = time.perf_counter()
        for circ in apps_cache["circs"]:
            ref.propagate(circ, obs, n_threads=cores, maxdegree=self.maxdeg, mincoeff=TAU, parallel="sharded")
        part = "" if self.cpu_steps == 20 else f" (first {self.cpu_steps} of 20 Trotter steps)"
        return sum(apps_cache["apps"]), time.perf_counter() - t0, cores, (
            f"the theta_h sweep of the same workload{part}, the reference built from its own sources, "
            f"parallel='sharded', n_threads={cores}")

    def serial_sample(self, min_seconds=6.0):
        """The oracle's serial port (one core, the reference's parallel="serial"
        strategy) on the first theta_h of the sweep, first serial_steps Trotter
        steps, repeated until min_seconds have passed."""
        from oracle import oracle as O
        keys, re, im = self.observable()
        tab = self.tables(self.serial_steps)[0]
        apps, runs = 0, 0
        t0 = time.perf_counter()
        while runs == 0 or time.perf_counter() - t0 < min_seconds:
            apps += O.pauli_propagate(tab, keys, re, im, maxdegree=self.maxdeg, mincoeff=TAU, n_threads=1).apps
            runs += 1
        part = "" if self.serial_steps == 20 else f", first {self.serial_steps} of 20 Trotter steps"
        return apps, time.perf_counter() - t0, (
            f"{runs} x theta_h={self.thetas[0]:.6g}{part}, serial port of the reference algorithm")

    def config(self):
        return {"workload": self.name, "lattice": "10x10 open", "trotter_steps": 20,
                "maxdegree": self.maxdeg, "mincoeff": TAU, "theta_h": [round(t, 6) for t in self.thetas],
                "observable": "Z_55", "batched": True}


class KickedIsingW10(KickedIsing):
    """The same circuit at maximum weight 10, theta_h = 0.3: the large-N case
    (about 4e8 terms inside a batch at the peak, 2e11 apps per propagation)."""
    name = "kicked_ising_10x10_w10_tau1e-6"
    metric = "term-gate applications/s (10x10 kicked Ising, 20 steps, W=10, tau=1e-6, theta_h=0.3)"
    thetas = (0.3,)
    maxdeg = 10
    cpu_steps = 9
    serial_steps = 3
    # the DRAM traffic of the W=8 capture does not carry over: at W=10 the
    # store (about 16 GB at its peak) is far larger than L2; not measured
    traffic = None
    traffic_note = "not measured at W=10 (a full-size multi-kernel capture is too large to profile)"


class Hubbard:
    """6x6 spinful Fermi-Hubbard in Majorana form (144 Majoranas), 10 Trotter steps,
    t=1, U=4, dt=0.1, observable n_(0,up) = 0.5 (1 + i g0 g1), degree <= 6, tau = 1e-7."""
    name = "hubbard_6x6_10steps_deg6_tau1e-7"
    metric = "term-gate applications/s (6x6 Fermi-Hubbard Majorana, 10 steps, deg<=6, tau=1e-7)"
    kind = "majorana"
    bytes_per_term = 24 + 16  # 3 words of Majorana bits + complex FP64 coefficient
    kernel = "Majorana batch-orbit path (morbit_*) + persistent per-gate kernel for the first gate"
    launch_unit = "one commuting run (orbit batch)"
    steps = 10
    cpu_steps = 6
    params = dict(has_maxdegree=1, maxdegree=6, mincoeff=1e-7, deterministic=0)

    def _table(self, steps):
        import fastfermion_gb300 as ff
        return ff.encode_majorana_circuit(ff.build_circuit(ff.workloads.hubbard_circuit(6, 6, steps=steps)))

    def tables(self):
        return [self._table(self.steps)]

    def observable(self):
        keys = np.zeros((4, 2), dtype=np.uint64)
        keys[0, 1] = 3  # g0 g1
        return keys, np.array([0.5, 0.0]), np.array([0.0, 0.5])

    def propagate(self, ctx, k, re, im, tab, n=None):
        p = dict(self.params)
        if n is not None:
            p["n"] = n
        return ctx.majorana_propagate(k, re, im, tab, p, on_device=n is not None)

    def cpu_sample(self, tabs, cores, min_seconds=0.0):
        """The oracle's serial port (the reference's Majorana path is serial) on the
        first cpu_steps Trotter steps (about 15 s of one core)."""
        from oracle import oracle as O
        keys, re, im = self.observable()
        tab = self._table(self.cpu_steps)
        t0 = time.perf_counter()
        r = O.majorana_propagate(tab, keys, re, im, maxdegree=6, mincoeff=1e-7)
        return r.apps, time.perf_counter() - t0, 1, (
            f"the first {self.cpu_steps} of 10 Trotter steps, serial port of the reference "
            "algorithm (the reference's Majorana path has no parallel strategy)")

    def config(self):
        return {"workload": self.name, "lattice": "6x6 open, spinful (144 Majoranas)",
                "trotter_steps": self.steps, "t": 1.0, "U": 4.0, "dt": 0.1, "maxdegree": 6,
                "mincoeff": 1e-7, "observable": "0.5 (1 + i g0 g1)"}


class BatchedAnsatz:
    """256 instances of a 50-qubit open-chain hardware-efficient ansatz (8 layers of
    RY on every qubit then CZ on the bonds), per-instance angles from uniform[-pi, pi]
    and per-instance observables of 1..64 random weight-1..4 terms, W = 6,
    tau = 1e-7.  One step = one batched propagation of all 256 instances with
    checkpoints, then the adjoint gradient d<O_i>/dtheta of all 400 angles of
    every instance."""
    name = "hea_50q_8layers_256inst_w6_tau1e-7"
    metric = ("term-gate applications/s (256-instance 50-qubit ansatz, W=6, tau=1e-7; "
              "forward + adjoint gradient per step)")
    kind = "batched"
    ninst, nq, layers = 256, 50, 8
    cpu_instances = 96

    def tables(self):
        import fastfermion_gb300 as ff
        from fastfermion_gb300 import workloads as W
        self.thetas, self.obs = W.hea_instances(self.ninst, n=self.nq, layers=self.layers)
        self.keys = np.concatenate([o[0] for o in self.obs], axis=1)
        self.re = np.concatenate([o[1] for o in self.obs])
        self.off = np.cumsum([0] + [o[1].size for o in self.obs]).astype(np.int64)
        return [ff.encode_pauli_circuit(ff.build_circuit(W.hea_circuit(self.nq, self.layers)))]

    def params(self):
        return dict(maxdegree=6, topk=0, mincoeff=1e-7, max_xweight=-1, xtrunc_period=1, batched=1,
                    deterministic=0)

    def cpu_sample(self, tabs, cores, min_seconds=0.0):
        """The oracle's sharded OpenMP port of the reference, instance by instance
        (the reference has no batching), on the first cpu_instances instances."""
        from oracle import oracle as O
        tab = tabs[0]
        apps = 0
        t0 = time.perf_counter()
        for i in range(self.cpu_instances):
            t = tab.copy()
            t["theta"][t["kind"] == 0] = self.thetas[i]
            k, r = self.obs[i]
            apps += O.pauli_propagate(t, k, r, np.zeros(r.size), maxdegree=6, mincoeff=1e-7,
                                      n_threads=cores).apps
        return apps, time.perf_counter() - t0, cores, (
            f"the first {self.cpu_instances} of 256 instances, forward only, one at a time, sharded "
            "OpenMP port of the reference algorithm (the reference has no gradient)")

    def config(self):
        return {"workload": self.name, "instances": self.ninst, "qubits": self.nq, "layers": self.layers,
                "angles_per_instance": self.nq * self.layers, "maxdegree": 6, "mincoeff": 1e-7,
                "observables": "1..64 random terms of weight 1..4, N(0,1) coefficients",
                "checkpoint_every": 1}


class LearnedCorrection:
    """Learned truncation correction on the 10x10 kicked-Ising circuit (20 steps,
    observable Z_55, threshold 1e-6): plain W=6 propagation plus the surrogate's
    correction, judged against plain W'=10.  Training: 64 seeded theta_h values
    in [0.05, pi/2]; evaluation: 16 held-out values from the same range.  The
    line's value is the time to reach |delta<O>| <= 1e-3 on the 16 held-out
    values (seconds, summed): the surrogate path (W=6 with capture, features,
    network; plus the W'=10 fallback where its error exceeds the bound),
    against the cheapest plain propagation within the bound."""
    name = "learned_correction_kicked_ising_10x10_w6_to_w10"
    metric = ("time-to-|delta<O>|<=1e-3 on 16 held-out theta_h (s), surrogate-corrected W=6 "
              "(fallback to plain W=10 where it misses) vs plain")
    kind = "surrogate"
    members, steps, lr = 2, 20000, 3e-3

    def config(self):
        return {"workload": self.name, "lattice": "10x10 open", "trotter_steps": 20, "maxdegree": 6,
                "judge_maxdegree": 10, "mincoeff": 1e-6, "observable": "Z_55", "train_theta_h": 64,
                "held_out_theta_h": 16, "network": "32-128-128-128-1 GELU, BF16 tcgen05 GEMMs, FP32 accumulation",
                "ensemble": self.members, "train_steps": self.steps}


WORKLOADS = {"kicked_ising": KickedIsing, "kicked_ising_w10": KickedIsingW10, "hubbard": Hubbard,
             "surrogate": LearnedCorrection, "hea": BatchedAnsatz}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="kicked_ising", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-roofline", action="store_true")
    ap.add_argument("--sweep", default="batched", choices=["separate", "batched"],
                    help="Pauli workloads: one propagation per theta_h (separate), or all theta_h as "
                         "instances of one batched propagation with per-instance angles (batched)")
    ap.add_argument("--thetas", default=None,
                    help="comma-separated subset of theta_h (profiling runs; not a bench line)")
    a = ap.parse_args()
    a.wl = WORKLOADS[a.workload]()
    if a.thetas:
        a.wl.thetas = tuple(float(t) for t in a.thetas.split(","))
    return a


# ---------------------------------------------------------------------------
# distributed plumbing (replicas)
# ---------------------------------------------------------------------------
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return rank, ws, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"ffg_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                rows.append((float(p[1]), float(p[2]), p[5], p[6], p[7], p[8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        reasons = set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            for name, v in zip(names, r[2:]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "samples": len(rows), "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# CPU baseline (the oracle's port of the reference algorithm)
# ---------------------------------------------------------------------------
def cpu_baseline(wl, tabs):
    """The reference itself (built from its own sources in baseline/_ref) where
    the workload has a reference sample and the build exists, else the oracle's
    port; about 10 s of host time."""
    cores = os.cpu_count() or 1
    ref = reference_module() if hasattr(wl, "ref_sample") else None
    if ref is not None:
        cache, apps, dt = {}, 0, 0.0
        while dt < 10.0:
            a, t, cores, desc = wl.ref_sample(ref, cores, cache)
            apps += a
            dt += t
        kind = "reference"
    else:
        apps, dt, cores, desc = wl.cpu_sample(tabs, cores, min_seconds=10.0)
        kind = "port"
    out = {"value": apps / dt, "unit": UNIT, "cores": cores, "kind": kind,
           "sample": f"{desc} ({apps} apps, {dt:.1f} s)"}
    if hasattr(wl, "serial_sample"):
        apps, dt, desc = wl.serial_sample()
        out["serial"] = {"value": apps / dt, "unit": UNIT, "cores": 1,
                         "sample": f"{desc} ({apps} apps, {dt:.1f} s)"}
    return out


def reference_module():
    """The reference package built from its own sources into baseline/_ref (by
    oracle/ref.mk from the staged copy), or None where it is not built."""
    import glob
    stage = os.path.join(ROOT, "baseline", "_ref")
    if not glob.glob(os.path.join(stage, "fastfermion", "ffcore*.so")):
        return None
    if stage not in sys.path:
        sys.path.insert(0, stage)
    try:
        import fastfermion
        return fastfermion
    except Exception:
        return None


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    wl = args.wl
    if wl.kind == "surrogate":
        print(json.dumps({"impl": "reference", "unavailable": (
            "the reference reaches 1e-3 only by plain W=10, hours on the host for the 16 held-out theta_h "
            "(986 s at theta_h=0.3 alone); a bounded sample of it is the cpu_baseline of the GPU line")}))
        return 0
    from oracle import oracle as O
    O.build()
    tabs = wl.tables()
    cores = os.cpu_count() or 1
    ref = reference_module() if hasattr(wl, "ref_sample") else None
    if ref is not None:
        cache = {}
        sample = lambda: wl.ref_sample(ref, cores, cache)  # noqa: E731
        kind = "reference"
    else:
        sample = lambda: wl.cpu_sample(tabs, cores)  # noqa: E731
        kind = "port"
    for _ in range(args.warmup):
        sample()
    tot, dt = 0, 0.0
    for _ in range(args.steps):
        apps, t, cores, desc = sample()
        tot += apps
        dt += t
    v = tot / dt
    print(json.dumps({
        "impl": "reference", "metric": wl.metric, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": wl.config(),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"{desc}, per step"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
    return 0


# ---------------------------------------------------------------------------
# GPU arm, batched ansatz (forward + adjoint through the public C ABI)
# ---------------------------------------------------------------------------
def main_batched(args, rank, ws, local, dist):
    import torch

    from fastfermion_gb300 import _native
    torch.cuda.set_device(local)
    ctx = _native.context(local)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    wl = args.wl
    tabs = wl.tables()
    l2 = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    w = np.ones(wl.ninst)

    def step():
        expect, h = ctx.pauli_propagate_batched(wl.keys, wl.re, wl.off, tabs[0], wl.thetas, wl.params(), 1)
        pr = ctx.profile()
        t1 = time.perf_counter()
        g, _ = h.adjoint(w)
        t_adj = time.perf_counter() - t1
        h.free()
        step.emits = pr["emits"]
        return pr["apps"], pr["kernel_launches"], pr["seconds_total"], t_adj, expect, g

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(dist)
    times, host_times, apps_tot, launches, fwd_s, adj_s = [], [], 0, 0, 0.0, 0.0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            l2.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            t0 = time.perf_counter()
            e0.record(stream)
            a, nl, tf, ta, _, _ = step()
            e1.record(stream)
            e1.synchronize()
            host_times.append(time.perf_counter() - t0)
            times.append(e0.elapsed_time(e1) * 1e-3)
            apps_tot += a
            launches += nl
            fwd_s += tf
            adj_s += ta
    barrier(dist)
    t_max = allmax(dist, sum(times))
    value = allsum(dist, apps_tot) / t_max
    e2e = allsum(dist, apps_tot) / allmax(dist, sum(host_times))
    cpu = cpu_baseline(wl, tabs) if rank == 0 and not args.no_cpu_baseline else None
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm_peak = json.load(open(pk)).get("hbm_gbs", 6800.0) if os.path.exists(pk) else 6800.0
    if rank == 0:
        k = args.steps
        h2d = wl.keys.nbytes + wl.re.nbytes + wl.off.nbytes + wl.thetas.nbytes + tabs[0].nbytes
        d2h = wl.ninst * 8 + wl.thetas.nbytes
        print(json.dumps({
            "metric": wl.metric, "value": value, "unit": UNIT, "n_gpus": ws, "steps": k, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_max / k, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": dict(wl.config(), apps_per_step=apps_tot / k, forward_ms=1e3 * fwd_s / k,
                           adjoint_ms=1e3 * adj_s / k, l2="flushed between steps (512 MB write)",
                           parallelism=f"replicas{ws}",
                           inputs="host arrays (the batched entry point copies them in each step)"),
            "roofline": (lambda ab: {
                "bound": "hbm", "achieved": ab / (t_max / k) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "frac": ab / (t_max / k) / 1e9 / hbm_peak, "traffic": None,
                "kernel": "orbit engine forward + adjoint kernels", "launch_unit": "one step (forward + adjoint)",
                "achieved_kind": "per-gate-equivalent of the forward pass (24 B x (2 x apps + emitted partners): "
                                 "16 B one-word x/z key + 8 B coefficient) over the whole step, the adjoint's time "
                                 "included; the engine keeps groups in shared memory and does not move these bytes",
                "algorithmic_bytes_per_step": ab})(24.0 * (2 * apps_tot / k + step.emits)),
            "cpu_baseline": cpu,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "clocks": clk.summary(),
            "gpu_launches": launches,
        }))
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
# ---------------------------------------------------------------------------
# learned correction (time to accuracy)
# ---------------------------------------------------------------------------
MLP_FLOPS_PER_ROW = 2 * (32 * 128 + 2 * 128 * 128 + 128)


def mlp_roofline(ctx, mlp, rows=1 << 21, reps=10):
    """Achieved TFLOP/s of the network's forward kernel (mlp_forward_kernel) on
    `rows` synthetic BF16 inputs, CUDA events on the context's stream."""
    import torch
    x = (torch.randn(rows, 32, device="cuda") * 0.5).to(torch.bfloat16).view(torch.int16)
    y = torch.empty(rows, dtype=torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(ctx.stream())
    for _ in range(3):
        mlp.forward(x, rows, y)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        mlp.forward(x, rows, y)
    e1.record(stream)
    e1.synchronize()
    sec = e0.elapsed_time(e1) * 1e-3 / reps
    return MLP_FLOPS_PER_ROW * rows / sec / 1e12, sec


def main_surrogate(args, rank, ws, local, dist):
    import torch

    from fastfermion_gb300 import _native, surrogate as S, workloads as W
    torch.cuda.set_device(local)
    ctx = _native.context(local)
    wl = S.kicked_ising_workload()
    train, held = W.learned_correction_thetas()
    t0 = time.perf_counter()
    sur = S.Surrogate(ctx, wl, seed=0, members=args.wl.members)
    data = sur.collect(train)
    t_data = time.perf_counter() - t0
    sur.fit(data, steps=args.wl.steps, lr=args.wl.lr)
    hdata = sur.collect(held)
    errs = sur.validate(hdata)
    for _ in range(args.warmup):
        sur.predict(held[0])
    with ClockSampler(local) as clk:
        rows = S.evaluate(sur, hdata)
        reps = []
        for _ in range(max(args.steps - 1, 0)):  # more timings of the prediction path
            reps.append([sur.predict(s.theta)[1] for s in hdata])
    t_pred = np.median(np.array([[r["t_predict"] for r in rows]] + reps), axis=0)
    # kernels of one query: the capture propagation's, the feature kernel, and a
    # forward pass and a reduction per ensemble member
    sur.predict(held[0])
    launches = sum(ctx.profile()["kernel_launches"] + 1 + 2 * args.wl.members for _ in rows)
    h2d = sum(wl.table(s.theta)[0].nbytes + 48 for s in hdata)  # gate table + observable per query
    d2h = 16 * len(hdata)  # the value and the record size
    t_sur = sum(tp + (r["t_judge"] if r["err_surrogate"] > 1e-3 else 0.0) for tp, r in zip(t_pred, rows))
    t_plain = sum(r["t_plain"] for r in rows)
    tflops, t_fwd = mlp_roofline(ctx, sur.mlp)
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    peak = peaks.get("bf16_tflops", 1900.0)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        ref = reference_module()
        sub = sorted(hdata, key=lambda s: s.judge_seconds)[:4]  # the quickest judge runs
        if ref is not None:
            from fastfermion_gb300 import workloads as WL
            obs = ref.poly(f"Z{OBS_SITE}")
            tr = 0.0
            for s in sub:
                circ = [ref.ROT(g[1], list(g[2]), g[3]) for g in WL.kicked_ising_circuit(s.theta)]
                a = time.perf_counter()
                ref.propagate(circ, obs, n_threads=os.cpu_count(), maxdegree=10, mincoeff=1e-6, parallel="sharded")
                tr += time.perf_counter() - a
            cpu = {"value": tr, "unit": "s", "cores": os.cpu_count(), "kind": "reference",
                   "sample": "plain W=10 (the only plain cutoff within 1e-3 where W=6 misses) on the 4 held-out theta_h "
                             f"with the quickest GPU judge runs ({', '.join(f'{s.theta:.3f}' for s in sub)}); the GPU "
                             f"judge takes {sum(s.judge_seconds for s in sub):.3f} s on them"}
    if rank == 0:
        within = int(sum(r["err_surrogate"] <= 1e-3 for r in rows))
        within_plain = int(sum(r["err_plain_w"] <= 1e-3 for r in rows))
        out = {
            "metric": args.wl.metric, "value": t_sur, "unit": "s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_sur, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 network, f64 propagation", "data": "synthetic",
            "config": dict(args.wl.config(), plain_seconds=t_plain, speedup_vs_plain=t_plain / t_sur,
                           held_out_within_1e3_surrogate=within, held_out_within_1e3_plain_w6=within_plain,
                           held_out_max_error=float(errs.max()), validated_path="surrogate" if
                           sur.held_out_error <= 1e-3 else "fallback (validated error above 1e-3)",
                           data_seconds=t_data, train_seconds=sur.train_seconds, train_rows=sur.rows,
                           per_theta=[{k: (round(v, 6) if isinstance(v, float) else v) for k, v in r.items()}
                                      for r in rows], l2="not flushed (per-query latency)"),
            "roofline": {"bound": "tensor", "achieved": tflops, "peak": peak, "unit": "TFLOP/s",
                         "frac": tflops / peak, "traffic": None,
                         "kernel": "mlp_forward_kernel (3 tcgen05 BF16 GEMMs per 128-row tile)",
                         "launch_unit": "forward pass over 2^21 synthetic rows",
                         "algorithmic_flops": f"{MLP_FLOPS_PER_ROW} per row", "launch_seconds": t_fwd,
                         "peak_source": "MEASURED_PEAKS.json bf16_tflops (of measured)" if peaks else "fallback"},
            "cpu_baseline": cpu,
            "e2e": {"value": t_sur, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "note": "every timed query starts from host arrays and returns the value to the host"},
            "clocks": clk.summary(),
            "gpu_launches": launches,
        }
        print(json.dumps(out))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    rank, ws, local, dist = dist_init()
    if args.wl.kind == "batched":
        return main_batched(args, rank, ws, local, dist)
    if args.wl.kind == "surrogate":
        return main_surrogate(args, rank, ws, local, dist)
    import torch

    import fastfermion_gb300 as ff  # noqa: F401
    from fastfermion_gb300 import _native
    torch.cuda.set_device(local)
    ctx = _native.context(local)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    wl = args.wl
    tabs = wl.tables()
    hk, hre, him = wl.observable()
    dk = torch.from_numpy(hk.astype(np.int64)).cuda()
    dre = torch.from_numpy(hre).cuda()
    dim = torch.from_numpy(him).cuda()
    l2 = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 512 MB > L2
    torch.cuda.synchronize()

    batched_sweep = args.sweep == "batched" and wl.kind == "pauli" and len(tabs) > 1
    if batched_sweep:
        # every theta_h as an instance with its own angles: the same terms,
        # bit for bit, as the separate propagations (ffg_pauli_propagate_batched)
        bk = np.repeat(hk, len(tabs), axis=1)
        bre = np.repeat(hre, len(tabs))
        boff = np.arange(len(tabs) + 1, dtype=np.int64) * hre.size
        bth = np.stack([t["theta"][t["kind"] == 0] for t in tabs])
        bparams = dict(wl.params)

    def step_device(profiling=False):
        ctx.set_profiling(profiling)
        apps, emits, launches, rot_s, nrot = 0, 0, 0, 0.0, 0
        if batched_sweep:
            _, h = ctx.pauli_propagate_batched(bk, bre, boff, tabs[0], bth, bparams, 0)
            pr = ctx.profile()
            h.free()
            return pr["apps"], pr["emits"], pr["kernel_launches"], pr["seconds_rotations"], pr["n_gates"]
        for tab in tabs:
            r = wl.propagate(ctx, dk.data_ptr(), dre.data_ptr(), dim.data_ptr(), tab, n=hre.size)
            pr = ctx.profile()
            apps += pr["apps"]
            emits += pr["emits"]
            launches += pr["kernel_launches"]
            rot_s += pr["seconds_rotations"]
            nrot += pr["n_gates"]
            r.free()
        return apps, emits, launches, rot_s, nrot

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    barrier(dist)
    times, apps_tot, emits_tot, launches_tot = [], 0, 0, 0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            l2.fill_(1.0)  # flush L2 between steps (not timed)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            a, em, nl, _, _ = step_device()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
            apps_tot += a
            emits_tot += em
            launches_tot += nl
    torch.cuda.synchronize()
    barrier(dist)
    t_local = sum(times)
    t_max = allmax(dist, t_local)
    apps_all = allsum(dist, apps_tot)
    value = apps_all / t_max

    # the same sweep as one propagation per theta_h, for comparison (not the value)
    separate = None
    if batched_sweep and not args.no_e2e:
        batched_sweep = False
        ts = []
        for _ in range(2):
            l2.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            a_sep = step_device()[0]
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        separate = a_sep / min(ts)
        batched_sweep = True

    # roofline: the per-gate algorithm's bytes (B_g = (S + 8)(2 N_g + E_g) summed
    # over the rotations of a step) over the same unprofiled CUDA-event step time
    # as `value`.  The orbit engine does not move those bytes (groups live in
    # shared memory, the store stays in L2), so this is a per-gate-equivalent
    # bandwidth; the physical DRAM traffic is reported beside it.
    alg_bytes_step = wl.bytes_per_term * (2 * apps_tot + emits_tot) / args.steps
    traffic = getattr(wl, "traffic", None)
    traffic_note = getattr(wl, "traffic_note", None)
    if batched_sweep and hasattr(wl, "dram_per_batched_step") and len(tabs) == 7:
        traffic, traffic_note = wl.dram_per_batched_step, wl.batched_traffic_note
    t_step = t_local / args.steps
    achieved = None if args.no_roofline else alg_bytes_step / t_step / 1e9
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    peak = peaks.get("hbm_gbs", 6800.0)

    # end-to-end through the public C ABI with host buffers
    ctx.set_profiling(False)
    e2e_times, h2d, d2h = [], 0, 0
    for _ in range(0 if args.no_e2e else max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        if batched_sweep:
            expect, h = ctx.pauli_propagate_batched(bk, bre, boff, tabs[0], bth, bparams, 0)
            keys, re, inst = h.copy()
            h.free()
            d2h += keys.nbytes + re.nbytes + inst.nbytes + expect.nbytes
            h2d += bk.nbytes + bre.nbytes + boff.nbytes + bth.nbytes + tabs[0].nbytes
            e2e_times.append(time.perf_counter() - t0)
            continue
        for tab in tabs:
            r = wl.propagate(ctx, hk, hre, him, tab)
            keys, re, im = r.copy()
            r.overlapwithzero() if wl.kind == "pauli" else r.fock_state(0, 0)
            d2h += keys.nbytes + re.nbytes + im.nbytes
            h2d += hk.nbytes + hre.nbytes + him.nbytes + tab.nbytes
            r.free()
        e2e_times.append(time.perf_counter() - t0)
    n_e2e = max(len(e2e_times), 1)
    e2e_value = (allsum(dist, apps_tot / args.steps * n_e2e) / allmax(dist, sum(e2e_times))
                 if e2e_times else None)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl, tabs)

    if rank == 0:
        out = {
            "metric": wl.metric, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(wl.config(), apps_per_step=apps_tot / args.steps, sweep=args.sweep,
                           sweep_note=("all theta_h as instances of one batched propagation "
                                       "(ffg_pauli_propagate_batched, per-instance angles; each instance's terms "
                                       "bit-identical to its own propagation)") if batched_sweep else
                           "one propagation per theta_h (ffg_pauli_propagate)",
                           separate_propagations_apps_per_s=separate,
                           l2="flushed between steps (512 MB write)", parallelism=f"replicas{ws}"),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None,
                         "traffic": traffic,
                         "traffic_note": traffic_note,
                         "kernel": wl.kernel, "launch_unit": "one step (the whole workload), CUDA events "
                                                            "on the context stream, unprofiled",
                         "achieved_kind": "per-gate-equivalent: the bytes a per-gate pass would move, "
                                          "over the measured step time; the orbit engine moves far fewer "
                                          "(see traffic), it is bound by latency, not by HBM",
                         "algorithmic_bytes_per_step": alg_bytes_step,
                         "algorithmic_bytes": f"{wl.bytes_per_term} B x (2 x apps + emitted partners): "
                                              "per-gate model, summed over the rotations of a step",
                         "physical_dram_gbs": (traffic / t_step / 1e9) if traffic else None,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback"},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d // n_e2e,
                    "d2h_bytes_per_step": d2h // n_e2e},
            "clocks": clk.summary(),
            "gpu_launches": launches_tot,
        }
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
