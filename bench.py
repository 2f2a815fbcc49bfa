#!/usr/bin/env python
"""Benchmark: lightcone multigrid BAO reconstruction at 256^3 on GB300.

Workload (one step = one reconstruction, as examples/lightcone_mg.jl runs it):
  data 5e5 + randoms 5e6 FP32 points on a lightcone shell (r = 1000-1500 Mpc/h,
  RA 0-90 deg, Dec 0-45 deg), padded 256^3 mesh (box from setup_box(randoms,
  pad 25 Mpc/h): cell 5.96 Mpc/h), CIC, R = 15 Mpc/h, b = 2, f = 0.8, local LOS;
  paint both catalogs -> smooth -> normalise -> residual-driven solve of the
  multigrid operator until the relative residual is <= 1e-6 -> displacement ->
  shifted positions of the data (:sum) and of the randoms (:sum and :disp).
The solve starts three ways, each timed: "zero" (plain multigrid: V-cycles
with 2+2 red-black sweeps), "spectral" (FFT-preconditioned corrections with
the box's mean line of sight, V-cycles if they stall; the headline default)
and "learned" (the trained CNN guess, then as spectral).
Inputs are seeded synthetic catalogs with the shapes and distributions of the
UNIT lightcone mocks the reference benchmarks on (those files are not here).

`python bench.py --gpus N --steps K --warmup W` prints one JSON line.
`--impl reference` times the reference's CPU algorithm (a C/OpenMP + scipy.fft
restatement, see oracle/cpu_port.py) on the host cores instead.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "baorec.jl_gb300"))

METRIC = "recons/s at 1e-6 residual, learned-start MG vs plain MG, 256^3, one GB300"
UNIT = "recons/s"
FALLBACK_HBM_GBS = 6800.0
FALLBACK_BF16_TFLOPS = 1900.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mesh", type=int, default=256)
    ap.add_argument("--n-data", type=int, default=500_000)
    ap.add_argument("--rand-factor", type=int, default=10)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched box-mock measurement")
    ap.add_argument("--only-start", action="store_true", help="time only the --start solve (no other starts)")
    ap.add_argument("--no-kernels", action="store_true", help="skip the per-kernel roofline and paint timings")
    ap.add_argument("--batch-mocks", type=int, default=64)
    ap.add_argument("--no-scale512", dest="scale512", action="store_false",
                    help="skip the 512^3 measurements (lightcone run! and solve, large box)")
    ap.add_argument("--set-tune", default="",
                    help="after the autotuner, force choices: comma-separated key=value of pair_residual, acc_residual, "
                         "fft_zpass, fft_xy_fused, stream_residuals, tiles (per level, 1:1:0:0) (a profiler "
                         "distorts the tuner's timings, "
                         "so a launch list under ncu pins the choices of the timed run)")
    ap.add_argument("--conv-only", action="store_true",
                    help="only time the learned guess's tensor-core convolutions, every shape on a --mesh grid "
                         "(a small case for profilers)")
    ap.add_argument("--stencil-only", default="",
                    help="only time finest-level stencil kernels on a --mesh grid (a small case for profilers): "
                         "comma-separated kernel:pairs:acc[:xy], kernel 0 sweep, 1 accurate residual, 3 running "
                         "residual, 8 / 9 batched xy transform forward / inverse, pairs and acc the forms of "
                         "baorec_set_tune_pairs / baorec_set_tune_acc, xy 0 cuFFT or 1 the fused kernels")
    ap.add_argument("--stencil-reps", type=int, default=20)
    ap.add_argument("--paint-only", default="",
                    help="only time the CIC paint of the lightcone randoms into the --mesh grid (a small case "
                         "for profilers): comma-separated modes atomic, binned, deterministic")
    ap.add_argument("--start", default="spectral", choices=["zero", "spectral", "learned"],
                    help="start of the headline solve: zero (plain multigrid), spectral (FFT-preconditioned "
                         "corrections, V-cycles if they stall) or learned (CNN guess, then as spectral); "
                         "the other two are timed beside it under \"starts\"")
    return ap.parse_args()


def replica_seed(base, rank):
    """Each replica reconstructs its own mock: the base seed plus its rank."""
    return base + rank


def replica_throughput(ms, ws, dist=None, device="cuda"):
    """Replicas only (one reconstruction never shards): the slowest rank's
    time per step, taken over all ranks, and the whole job's reconstructions
    per second, ws of them per step.  Returns (ms_max, recons_per_s)."""
    if dist is not None and ws > 1:
        import torch
        t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, ws * 1000.0 / ms


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = []
        smax = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def measured_peak_tensor():
    """Dense BF16 tensor peak (TFLOP/s, burst: the convolution is timed alone)."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            return float(json.load(fh)["bf16_tflops"]), "measured"
    except Exception:
        return FALLBACK_BF16_TFLOPS, "fallback"


GUESS_CONV_SHAPES = ((8, 16, 256), (16, 16, 256), (32, 16, 256), (32, 32, 128), (64, 32, 128))


def guess_conv_rooflines(ctx, C, shapes=GUESS_CONV_SHAPES):
    """Tensor-core roofline of the learned guess's 3x3x3 convolutions: each
    tcgen05 shape of the network at its grid (256^3 level 0, 128^3 level 1)
    timed alone with CUDA events, beside the mma.sync kernel of the same shape."""
    peak, src = measured_peak_tensor()
    out = {}
    for cin, cout, n in shapes:
        row = {}
        for path, label in ((1, "tcgen05"), (2, "tcgen05_cpasync"), (0, "mma.sync")):
            avg, fl = C.c_float(), C.c_double()
            ctx.call("baorec_guess_profile_conv", cin, cout, n, path, 10, C.byref(avg), C.byref(fl))
            tf = fl.value / (avg.value * 1e-3) / 1e12
            row[label] = {"avg_launch_ms": avg.value, "achieved": tf}
        tc = row["tcgen05"]
        out[f"guess conv3 {cin}->{cout} at {n}^3"] = {
            "kernel": "conv_tc_kernel (tcgen05.mma, TMA slabs, TMEM accumulators)", "bound": "tensor",
            "achieved": tc["achieved"], "peak": peak, "unit": "TFLOP/s", "frac": tc["achieved"] / peak,
            "peak_source": src, "algorithmic_flops_per_launch": 2.0 * 27 * cin * cout * n ** 3,
            "avg_launch_ms": tc["avg_launch_ms"], "mma_sync": row["mma.sync"],
            "tcgen05_cpasync_loader": row["tcgen05_cpasync"]}
    return out


def power_timing(args, baorec, torch, np, X, R, bs, bm):
    """Yamamoto multipoles of the pre-reconstruction lightcone (data minus
    randoms, FKP weights with P0 = 5000 and the randoms' mean density as
    n(z), TSC, dk = 0.005) on the reconstruction mesh, device catalogs."""
    nd, nr = X[0].numel(), R[0].numel()
    omega = (np.pi / 2) * np.sin(np.radians(45.0))
    nbar = nd / (omega / 3 * (1500.0 ** 3 - 1000.0 ** 3))
    wf = 1.0 / (1.0 + nbar * 5000.0)
    wd = torch.full((nd,), wf, device="cuda")
    wr = torch.full((nr,), wf, device="cuda")
    rnz = torch.full((nr,), nbar, device="cuda")
    kw = dict(box_size=list(bs), box_min=list(bm), grid_size=args.mesh, mas="tsc", bin_size=0.005)
    baorec.power.compute_auto_lc(*X[:3], wd, None, *R[:3], wr, rnz, **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        res = baorec.power.compute_auto_lc(*X[:3], wd, None, *R[:3], wr, rnz, **kw)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / reps * 1e3
    mp = res["multipoles"]
    b = int(np.argmin(np.abs(res["k"] - 0.1)))
    return {"ms_per_call": ms, "particles": nd + nr, "mesh": args.mesh, "ffts": 22,
            "k_0.1": float(res["k"][b]), "P0_P2_P4_at_k_0.1": [float(v) for v in mp[b]],
            "note": "end to end through the Python API (host sums and result copy included)"}


def workload(args, seed):
    from baorec import mocks
    import numpy as np
    # the lognormal field is sampled on at most a 256^3 grid (above that, R = 15 Mpc/h smoothing leaves
    # less than 1e-3 of the power at its Nyquist wave number)
    m = mocks.lightcone_mock(n_data=args.n_data, rand_factor=args.rand_factor, n_grid=min(args.mesh, 256), seed=seed)
    # padded mesh: box from the randoms with a 25 Mpc/h pad (cell 5.96 Mpc/h at 256^3)
    pad = 25.0 * 256 / args.mesh
    f32 = np.float32
    bmin = np.array([m.rx.min(), m.ry.min(), m.rz.min()], f32) - f32(pad / 2)
    bmax = np.array([m.rx.max(), m.ry.max(), m.rz.max()], f32) + f32(pad / 2)
    side = f32(np.max(bmax - bmin))
    return m, [float(side)] * 3, [float(v) for v in bmin]


def batch_workload(count, seed):
    """Box mocks for the batched measurement: counts log-uniform in [1e5, 2e6],
    meshes alternating 128^3 (L = 1000 Mpc/h) and 256^3 (L = 2000 Mpc/h), CIC
    and TSC alternating in pairs, R uniform in [10, 15] Mpc/h.  Every catalog
    is Poisson-sampled (cell counts multinomial in 1 + δ, positions uniform in
    the cell, unit weights) from a lognormal field of the workload's P(k): one
    field per mesh size, moved periodically by a random number of cells per
    mock, so no two catalogs share a particle."""
    import numpy as np
    from baorec import mocks
    rng = np.random.default_rng(seed)
    fields = {128: (1000.0, mocks.lognormal_field(128, 1000.0, seed=seed)),
              256: (2000.0, mocks.lognormal_field(256, 2000.0, seed=seed + 1))}
    cdfs = {n: mocks.field_cdf(d) for n, (_, d) in fields.items()}
    out = []
    for i in range(count):
        n = 128 if i % 2 == 0 else 256
        L, delta = fields[n]
        npart = int(np.exp(rng.uniform(np.log(1e5), np.log(2e6))))
        x, y, z = mocks.sample_field(delta, npart, L, rng, shift=rng.integers(0, n, 3), cdf=cdfs[n])
        out.append(dict(x=x, y=y, z=z, w=np.ones(npart, np.float32), mesh=n, box_size=L,
                        mas="cic" if (i // 2) % 2 == 0 else "tsc", smoothing_radius=float(rng.uniform(10, 15))))
    return out


def run_batch(args, torch, np):
    """Batched box reconstructions (3 iterative-FFT steps each, LOS +z, :sum
    shifts) replayed as one CUDA graph; device-timed and end to end."""
    import baorec
    mk = batch_workload(args.batch_mocks, args.seed + 7)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    items, host_in, host_out, dev_in = [], [], [], []
    for m in mk:
        d = [dev(m[k]) for k in ("x", "y", "z", "w")]
        o = tuple(torch.empty(len(m["x"]), device="cuda") for _ in range(3))
        items.append(dict(x=d[0], y=d[1], z=d[2], w=d[3], mesh=m["mesh"], box_size=m["box_size"], mas=m["mas"],
                          smoothing_radius=m["smoothing_radius"], field="sum", out=o))
        host_in.append([torch.from_numpy(m[k]).pin_memory() for k in ("x", "y", "z", "w")])
        host_out.append([torch.empty(len(m["x"])).pin_memory() for _ in range(3)])
        dev_in.append(d)
    base = baorec.IterativeRecon(bias=2.0, f=0.8, smoothing_radius=15.0, los=[0.0, 0.0, 1.0], n_iter=3)
    t0 = time.perf_counter()
    b = baorec.Batch(base, items)
    t_build = time.perf_counter() - t0
    # the graph replays on a stream torch owns, so torch's copies and events never touch the library's
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        b.launch(sh)
    b.sync(sh)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        b.launch(sh)
    ev1.record(stream)
    b.sync(sh)
    ms = ev0.elapsed_time(ev1) / args.steps
    # end to end: inputs from pinned host memory, graph replay, shifted positions back
    with torch.cuda.stream(stream):
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for hi, di in zip(host_in, dev_in):
                for h, d in zip(hi, di):
                    d.copy_(h, non_blocking=True)
            b.launch(sh)
            for ho, it in zip(host_out, items):
                for h, d in zip(ho, it["out"]):
                    h.copy_(d, non_blocking=True)
        stream.synchronize()
        te = (time.perf_counter() - t0) / args.steps
    torch.cuda.synchronize()
    npart = sum(len(m["x"]) for m in mk)
    res = {"workload": f"{len(mk)} periodic box mocks, {npart} particles, meshes 128^3 (L=1000) / 256^3 (L=2000), "
                       "CIC/TSC, R 10-15, 3 iterative-FFT steps, LOS +z, :sum shifts, one CUDA graph",
           "value": len(mk) * 1000.0 / ms, "unit": "recons/s", "ms_per_batch": ms,
           "particles_per_s": npart * 1000.0 / ms, "graph_build_s": t_build,
           "gpu_launches_per_batch": b.kernel_launches(),
           "e2e": {"value": len(mk) / te, "unit": "recons/s", "h2d_bytes_per_step": 16 * npart,
                   "d2h_bytes_per_step": 12 * npart, "ms_per_step": te * 1e3}}
    b.close()
    return res


RUNNING_RESIDUAL = {
    0: "resid_kernel (difference form)",
    1: "resid_pairs_kernel (FP32 running residual, two z-adjacent cells per thread)",
    2: "resid_pairz_kernel (FP32 running residual, plane pairs streamed in z, 16-plane blocks)",
    3: "resid_pairz_kernel (FP32 running residual, plane pairs streamed in z, 32-plane blocks)",
    4: "resid_tma_kernel (FP32 running residual, TMA-staged, two x-adjacent cells per thread, 32-plane columns)",
    5: "resid_tma_kernel (FP32 running residual, TMA-staged, two x-adjacent cells per thread, 16-plane columns)",
    6: "resid_pairs_kernel (FP32 running residual, two z-adjacent cells per thread, 32x8x16 tiles)",
}


def traffic_per_launch(name, N):
    """DRAM bytes per launch of `name` from the committed ncu capture, scaled to N cells."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as fh:
            t = json.load(fh)[name]
        return t["dram_bytes"] * N / t["cells"]
    except Exception:
        return None


def run_box(args, torch, np):
    """The periodic-box workload: 2e5 particles Poisson-sampled from the
    lognormal field, 128^3 mesh, L = 1000 Mpc/h, CIC, R = 15, b = 2, f = 0.8,
    LOS +z, 3 iterative-FFT steps, shifted positions (:sum); device arrays,
    CUDA events on the context stream.  Returns the timing and the context
    (its result is the last reconstruction)."""
    import baorec
    from baorec import _lib, mocks
    n, L = 128, 1000.0
    m = mocks.box_mock(n_part=200_000, L=L, n_grid=n, seed=1234)
    rec = baorec.IterativeRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=[L] * 3, box_min=[0.0] * 3,
                                los=[0.0, 0.0, 1.0], n_iter=3)
    ctx = baorec.setup_fft_(rec, (n,) * 3)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    X = [dev(a) for a in (m.x, m.y, m.z, m.w)]
    out = [torch.empty(len(m.x), device="cuda") for _ in range(3)]
    ptrs = [t.data_ptr() for t in X]
    optr = [t.data_ptr() for t in out]
    torch.cuda.synchronize()

    def step():
        ctx.call("baorec_reconstructed_overdensity", *ptrs, len(m.x), None, None, None, None, 0, _lib.ASYNC)
        ctx.call("baorec_reconstructed_positions", *ptrs[:3], len(m.x), _lib.FIELD["sum"], *optr, _lib.ASYNC)

    for _ in range(args.warmup):
        step()
    stream = torch.cuda.ExternalStream(ctx.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    return {"workload": "periodic box 128^3, L=1000, 2e5 particles, CIC, R=15, b=2, f=0.8, LOS +z, 3 iterations, "
                        ":sum shifted positions", "value": 1000.0 / ms, "unit": "recons/s", "ms_per_step": ms}, \
        (m, rec, ctx)


def _events_ms(torch, stream, fn, reps):
    """Mean device time of fn() between CUDA events on `stream` (after one untimed call)."""
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def run_scale_512(args, torch, np, checks):
    """The reference's own scale: every number it publishes is at 512^3
    (test/benchmarks_gpu.out:9,25,45,61; test/benchmarks_cpu.out:6,12).

    lightcone: the headline catalogs (5e5 data + 5e6 randoms) on a 512^3 mesh.
      * run! as test/benchmarks_gpu.jl:116-160 times it (randoms, so the box is
        setup_box(randoms, 500); local line of sight): the iterative method
        with 3 iterations and the multigrid method with the reference's FMG
        schedule, each followed by reconstructed_positions of the data (:sum).
        With the catalog's observer inside that box, a 4^3 cell centre of the
        FMG hierarchy falls within 0.01 Mpc/h of it and the schedule's
        coefficient g = β/|x|^2 overflows (NaN in FP32 on any device), so
        these runs move the catalog by +100 Mpc/h on every axis; the
        residual-driven solver clamps those cells and needs no such move.
      * the residual-driven solve to 1e-6 with the FFT start on the
        headline's box with the pad scaled to the mesh (setup_box(randoms,
        12.5), cell 2.95 Mpc/h), through the
        C ABI: device recons/s, end to end with pinned host catalogs, the
        dominant kernel's roofline and the FP64 displacement error.
    large_box (the large-box workload): L = 3000 Mpc/h, 512^3, 2e7 particles
      from the lognormal field, TSC, R = 15, b = 2, f = 0.8, LOS +z: 5
      iterative-FFT steps, then the residual-driven multigrid solve with the
      learned start (network on the 256^3 restriction); shifted positions
      (:sum) after each.
    """
    import baorec
    from baorec import _lib, guess, mocks
    out = {}
    n5 = (512,) * 3
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    ptrs = lambda ts: [t.data_ptr() for t in ts]
    reps = max(2, min(args.steps, 5))
    # ---- lightcone at 512^3
    a5 = argparse.Namespace(**vars(args))
    a5.mesh = 512
    m, bs, bm = workload(a5, args.seed)
    nd, nr = len(m.x), len(m.rx)
    shift = np.float32(100.0)
    Xs = [dev(a + shift) for a in (m.x, m.y, m.z)] + [dev(m.w)]
    Rs = [dev(a + shift) for a in (m.rx, m.ry, m.rz)] + [dev(m.rw)]
    od = [torch.empty(nd, device="cuda") for _ in range(3)]
    SUM, DISP = _lib.FIELD["sum"], _lib.FIELD["disp"]
    ref_runs = {}
    for name, rec in (("iterative run! (3 iterations)", baorec.IterativeRecon(bias=2.0, f=0.8, smoothing_radius=15.0,
                                                                             n_iter=3, box_size=bs, box_min=bm)),
                      ("multigrid run! (reference FMG schedule)", baorec.MultigridRecon(
                          bias=2.0, f=0.8, smoothing_radius=15.0, box_size=bs, box_min=bm))):
        ctx = baorec.setup_fft_(rec, n5)
        stream = torch.cuda.ExternalStream(ctx.stream)
        run = lambda: ctx.call("baorec_run", *ptrs(Xs), nd, *ptrs(Rs), nr, 0)
        t_run = _events_ms(torch, stream, run, reps)
        read = lambda: ctx.call("baorec_reconstructed_positions", *ptrs(Xs[:3]), nd, SUM, *ptrs(od), _lib.ASYNC)
        t_read = _events_ms(torch, stream, read, reps)
        finite = bool(torch.isfinite(od[0]).all().item())
        ref_runs[name] = {"run_ms": t_run, "read_positions_ms": t_read, "finite": finite}
        ctx.close()
        rec.fft_plan = None
    ref_runs["reference_published"] = {"iterative run!": 595.8, "multigrid run!": 1820.0,
                                       "iterative read positions": 52.0, "multigrid read positions": 43.8,
                                       "unit": "ms", "hardware": "NERSC Perlmutter GPU node (model not stated)",
                                       "catalog": "UNIT ELG NGC lightcone, 0.8 < z < 1 (not available here)",
                                       "source": "test/benchmarks_gpu.out:9,25,45,61"}
    out["lightcone_run_512"] = ref_runs
    # residual-driven solve to 1e-6 on the headline box at 512^3
    X = [dev(a) for a in (m.x, m.y, m.z, m.w)]
    R = [dev(a) for a in (m.rx, m.ry, m.rz, m.rw)]
    rec = baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=bs, box_min=bm, los=None,
                                mg_mode="convergent", rtol=1e-6, start="spectral")
    ctx = baorec.setup_fft_(rec, n5)
    ctx.autotune(paint=False)
    ors, ori = [torch.empty(nr, device="cuda") for _ in range(3)], [torch.empty(nr, device="cuda") for _ in range(3)]

    def step(flags=0, xs=None, rs=None, o1=None, o2=None, o3=None):
        st = ctx.status("baorec_reconstructed_potential", *(xs or ptrs(X)), nd, *(rs or ptrs(R)), nr, flags)
        if st != _lib.OK:
            _lib.check(ctx.h, st)
        ctx.call("baorec_reconstructed_positions", *(xs or ptrs(X))[:3], nd, SUM, *(o1 or ptrs(od)), flags | _lib.ASYNC)
        ctx.call("baorec_reconstructed_positions2", *(rs or ptrs(R))[:3], nr, SUM, *(o2 or ptrs(ors)), DISP,
                 *(o3 or ptrs(ori)), flags)

    stream = torch.cuda.ExternalStream(ctx.stream)
    ms = _events_ms(torch, stream, step, reps)
    st = ctx.solve_stats()
    peak, src = measured_peak()
    avg, nbytes = ctypes.c_float(), ctypes.c_double()
    which = 5 if ctx.lib.baorec_tune_stream(ctx.h) != 0 else 3
    ctx.call("baorec_profile_kernel", which, 20, ctypes.byref(avg), ctypes.byref(nbytes))
    ach = nbytes.value / (avg.value * 1e-3) / 1e9
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    hX = [pin(a) for a in (m.x, m.y, m.z, m.w)]
    hR = [pin(a) for a in (m.rx, m.ry, m.rz, m.rw)]
    ho = [[torch.empty(k).pin_memory() for _ in range(3)] for k in (nd, nr, nr)]
    kw = dict(xs=ptrs(hX), rs=ptrs(hR), o1=ptrs(ho[0]), o2=ptrs(ho[1]), o3=ptrs(ho[2]))
    step(_lib.HOST, **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        step(_lib.HOST, **kw)
    torch.cuda.synchronize()
    te = (time.perf_counter() - t0) / reps
    lc = {"workload": f"lightcone 512^3 to 1e-6 relative residual (FFT start), {nd} data + {nr} randoms, "
                      "setup_box(randoms, 12.5)", "value": 1000.0 / ms, "unit": "recons/s", "ms_per_step": ms,
          "solver": {k: st[k] for k in ("cycles", "spectral_steps", "rel_residual")},
          "e2e": {"value": 1.0 / te, "unit": "recons/s", "ms_per_step": te * 1e3,
                  "h2d_bytes_per_step": 16 * (nd + nr) + 12 * nd + 12 * nr, "d2h_bytes_per_step": 12 * nd + 24 * nr},
          "roofline": {"kernel": (RUNNING_RESIDUAL[ctx.lib.baorec_tune_pairs(ctx.h)].split()[0] if which == 3
                                  else "resid_diff_stream_kernel") + " (finest level 512^3)", "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                       "frac": ach / peak, "peak_source": src, "avg_launch_ms": avg.value,
                       "algorithmic_bytes_per_launch": nbytes.value}}
    if checks:
        lc["l2_vs_fp64"] = _fp64_solve_check(torch, np, ctx, X, R, bs, bm, n5)
    out["lightcone_512"] = lc
    ctx.close()
    rec.fft_plan = None
    del X, R, Xs, Rs, hX, hR, ho, ors, ori
    torch.cuda.empty_cache()
    # ---- the large box
    bmock = mocks.box_mock(n_part=20_000_000, L=3000.0, n_grid=256, seed=args.seed + 11)
    nb = len(bmock.x)
    B = [dev(a) for a in (bmock.x, bmock.y, bmock.z, bmock.w)]
    ob = [torch.empty(nb, device="cuda") for _ in range(3)]
    box = dict(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=[3000.0] * 3, box_min=[0.0] * 3, los=[0.0, 0.0, 1.0],
               mas="tsc")
    rit = baorec.IterativeRecon(n_iter=5, **box)
    weights = os.path.join(ROOT, "baorec.jl_gb300", "weights", "guess_lightcone.npy")
    rmg = baorec.MultigridRecon(mg_mode="convergent", rtol=1e-6, start="learned", guess_params=guess.load_params(weights),
                                guess_level=1, **box)
    cit, cmg = baorec.setup_fft_(rit, n5), baorec.setup_fft_(rmg, n5)
    cmg.autotune(paint=False)

    def big_iter():
        cit.call("baorec_reconstructed_overdensity", *ptrs(B), nb, None, None, None, None, 0, _lib.ASYNC)
        cit.call("baorec_reconstructed_positions", *ptrs(B[:3]), nb, SUM, *ptrs(ob), _lib.ASYNC)

    def big_mg():
        s_ = cmg.status("baorec_reconstructed_potential", *ptrs(B), nb, None, None, None, None, 0, 0)
        if s_ != _lib.OK:
            _lib.check(cmg.h, s_)
        cmg.call("baorec_reconstructed_positions", *ptrs(B[:3]), nb, SUM, *ptrs(ob), 0)

    t_it = _events_ms(torch, torch.cuda.ExternalStream(cit.stream), big_iter, reps)
    t_mg = _events_ms(torch, torch.cuda.ExternalStream(cmg.stream), big_mg, reps)
    smg = cmg.solve_stats()
    lb = {"workload": "box L=3000, 512^3, 2e7 particles (lognormal, Poisson-sampled), TSC, R=15, b=2, f=0.8, LOS +z: "
                      "5 iterative-FFT steps, then the multigrid solve to 1e-6 with the learned start (network on the "
                      "256^3 restriction); :sum shifted positions after each",
          "value": 1000.0 / (t_it + t_mg), "unit": "recons/s", "ms_per_step": t_it + t_mg, "iterative_ms": t_it,
          "multigrid_ms": t_mg, "particles_per_s": nb * 1000.0 / (t_it + t_mg),
          "solver": {k: smg[k] for k in ("cycles", "spectral_steps", "rel_residual", "rel_residual_initial")}}
    if checks:
        lb["l2_vs_fp64"] = _fp64_large_box_check(torch, np, cit, cmg, B, n5)
    out["large_box_512"] = lb
    cit.close()
    cmg.close()
    return out


def _fp64_solve_check(torch, np, ctx, X, R, bs, bm, n):
    """Displacement error of the GPU's residual-driven solve at this size against
    the FP64 oracle solution of the same right-hand side."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import baorec
    import fp64_oracle as P
    # torch fills these on its own stream: finish that before the context's stream uses them
    fd, phi = baorec.zeros_mesh(n), baorec.zeros_mesh(n)
    g = [baorec.zeros_mesh(n) for _ in range(3)]
    torch.cuda.synchronize()
    ctx.call("baorec_setup_overdensity_randoms", fd.data_ptr(), *[t.data_ptr() for t in X], X[0].numel(),
             *[t.data_ptr() for t in R], R[0].numel(), 0)
    ctx.call("baorec_mg_solve", fd.data_ptr(), phi.data_ptr(), None, None)
    ctx.call("baorec_set_result", phi.data_ptr(), 0)
    ctx.call("baorec_displacement_meshes", *[t.data_ptr() for t in g])
    torch.cuda.synchronize()
    f_np = fd.cpu().numpy()
    beta = np.float32(np.float32(0.8) / np.float32(2.0))
    phi64, _, hist = P.solve(f_np, bs, bm, beta, None, rtol=1e-10)
    g64 = P.gradient_meshes(phi64, np.asarray(bs, np.float64))
    gs = P.gradient_meshes(phi.cpu().numpy().astype(np.float64), np.asarray(bs, np.float64))
    return {"displacement": P.rel_l2_vector([t.cpu().numpy() for t in g], g64),
            "solution": P.rel_l2_vector(gs, g64), "fp64_solve_rel_residual": hist[-1],
            "note": "displacement = the GPU's FP32-transform gradient; solution = the GPU potential differentiated "
                    "in FP64; both against the FP64 solution of the GPU's right-hand side"}


def _fp64_large_box_check(torch, np, cit, cmg, B, n):
    """The large box against FP64: the GPU's painted, smoothed, normalised
    overdensity is iterated 5 times by the FP64 oracle (src/iterative.jl) and
    solved by the FP64 operator; the displacement meshes of both GPU results
    are compared with those FP64 fields."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import baorec
    import baorec_oracle as O
    import fp64_oracle as P
    L = np.array([3000.0] * 3)
    d = baorec.zeros_mesh(n)
    g = [baorec.zeros_mesh(n) for _ in range(3)]
    phi = baorec.zeros_mesh(n)
    # torch fills these on its own stream: finish that before the contexts' streams use them; the paint
    # without BAOREC_WRITEBACK leaves the positions as they are
    torch.cuda.synchronize()
    cit.call("baorec_setup_overdensity", d.data_ptr(), *[t.data_ptr() for t in B[:3]], B[3].data_ptr(), B[0].numel(),
             1, 0)
    torch.cuda.synchronize()
    d64 = d.cpu().numpy().astype(np.float64)
    O.set_fft_workers(os.cpu_count())
    k = O.k_vec(n, L, np.float64)
    beta = np.float64(np.float32(np.float32(0.8) / np.float32(2.0)))
    dr = d64.copy()
    for it in range(1, 6):
        dr = O.iterate(dr, d64, k, it, beta, los=[0.0, 0.0, 1.0])
    psi64 = O.displacement_meshes_iterative(dr, L)
    cit.call("baorec_displacement_meshes", *[t.data_ptr() for t in g])
    torch.cuda.synchronize()
    it_err = P.rel_l2_vector([t.cpu().numpy() for t in g], psi64)
    del psi64, dr
    phi64, _, hist = P.solve(d64, L, np.zeros(3), np.float32(beta), [0.0, 0.0, 1.0], rtol=1e-10)
    g64 = P.gradient_meshes(phi64, L)
    cmg.call("baorec_mg_solve", d.data_ptr(), phi.data_ptr(), None, None)
    cmg.call("baorec_set_result", phi.data_ptr(), 0)
    cmg.call("baorec_displacement_meshes", *[t.data_ptr() for t in g])
    torch.cuda.synchronize()
    mg_err = P.rel_l2_vector([t.cpu().numpy() for t in g], g64)
    O.set_fft_workers(None)
    return {"iterative": it_err, "multigrid": mg_err, "fp64_solve_rel_residual": hist[-1],
            "note": "GPU displacement meshes against the FP64 oracle from the GPU's overdensity (the paint is "
                    "checked against the oracle at smaller sizes)"}


def oracle_checks(args, torch, np, ctxs, m, bs, bm, X, R, box):
    """Relative L2 error of the displacement field against the FP64 oracle
    (oracle/fp64_oracle.py, oracle/baorec_oracle.py) for both workloads,
    computed after the timed region on the host cores.

    Lightcone: the right-hand side the GPU painted and normalised is solved
    by every start's GPU solve and, in FP64, by the oracle; "solve" is the
    error of the GPU gradient against that FP64 gradient (the arithmetic of
    the solve and the gradient).  "pipeline" compares the same GPU gradient
    with the FP64 oracle run from the particles (paint, smoothing,
    normalisation and solve all in FP64); cells where the randoms' threshold
    test of src/recon.jl:86-88 comes out differently in FP32 and FP64 are
    counted in "threshold_flips".  Box: the GPU displacement meshes against
    the FP64 oracle run of the same catalog."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import baorec
    import baorec_oracle as O
    import fp64_oracle as P
    n = (args.mesh,) * 3
    beta = np.float32(np.float32(0.8) / np.float32(2.0))
    t0 = time.perf_counter()
    c0 = next(iter(ctxs.values()))
    fd = baorec.zeros_mesh(n)
    torch.cuda.synchronize()   # torch zero-fills on its own stream
    c0.call("baorec_setup_overdensity_randoms", fd.data_ptr(), *[t.data_ptr() for t in X], X[0].numel(),
            *[t.data_ptr() for t in R], R[0].numel(), 0)
    torch.cuda.synchronize()
    f_np = fd.cpu().numpy()
    grads = {}
    for start, c in ctxs.items():
        phi = baorec.zeros_mesh(n)
        g = [baorec.zeros_mesh(n) for _ in range(3)]
        torch.cuda.synchronize()
        st = c.status("baorec_mg_solve", fd.data_ptr(), phi.data_ptr(), None, None)
        c.call("baorec_set_result", phi.data_ptr(), 0)
        c.call("baorec_displacement_meshes", *[t.data_ptr() for t in g])
        torch.cuda.synchronize()
        grads[start] = ([t.cpu().numpy() for t in g], st, c.solve_stats()["rel_residual"])
    phi64, _, hist = P.solve(f_np, bs, bm, beta, None, rtol=1e-11)
    g64 = P.gradient_meshes(phi64, np.asarray(bs, np.float64))
    solve = {s: {"l2": P.rel_l2_vector(g, g64), "status": st, "rel_residual": rr} for s, (g, st, rr) in grads.items()}
    f64 = O.setup_overdensity_randoms(np.zeros(n, np.float64), 2.0, 15.0, np.asarray(bs, np.float64),
                                      np.asarray(bm, np.float64), m.x, m.y, m.z, m.w, m.rx, m.ry, m.rz, m.rw)
    flips = int(((f64 == 0) != (f_np == 0)).sum())
    phip, _, _ = P.solve(f64, bs, bm, beta, None, rtol=1e-11)
    gp = P.gradient_meshes(phip, np.asarray(bs, np.float64))
    pipeline = {s: P.rel_l2_vector(g, gp) for s, (g, _, _) in grads.items()}
    lc = {"solve": solve, "pipeline": pipeline, "threshold_flips": flips, "fp64_solve_rel_residual": hist[-1],
          "note": "GPU gradient of the potential vs the FP64 oracle; solve = same right-hand side, pipeline = "
                  "FP64 from the particles"}
    # box: displacement meshes of the last timed reconstruction vs the FP64 oracle run
    bm_, brec, bctx = box
    L = float(brec.box_size[0])
    nb = (bctx.cfg.n[0],) * 3
    # the timed steps painted the same catalog (positions inside the box, nothing wraps)
    psi = [baorec.zeros_mesh(nb) for _ in range(3)]
    torch.cuda.synchronize()
    bctx.call("baorec_displacement_meshes", *[t.data_ptr() for t in psi])
    torch.cuda.synchronize()
    d64, _, _, _ = O.run_iterative(nb, 2.0, 0.8, 15.0, bm_.x, bm_.y, bm_.z, bm_.w, box_size=[L] * 3,
                                   box_min=[0.0] * 3, los=[0.0, 0.0, 1.0], n_iter=3, dtype=np.float64)
    psi64 = O.displacement_meshes_iterative(d64, np.array([L] * 3))
    bx = {"l2": P.rel_l2_vector([t.cpu().numpy() for t in psi], psi64),
          "note": "GPU displacement meshes of the box reconstruction vs the FP64 oracle run"}
    return {"lightcone_%d" % args.mesh: lc, "box_128": bx, "seconds": time.perf_counter() - t0}


def cpu_baseline(args, m, bs, bm, reps=1, solver="fmg"):
    """The reference's CPU algorithm on this host: one full reconstruction per
    sample; solver "convergent" replaces its FMG schedule by the GPU's
    solver run to 1e-6 on the host."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from cpu_port import CpuPort
    port = CpuPort()
    n = (args.mesh,) * 3
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        port.lightcone_reconstruction(m, n, bs, bm, solver=solver)
        times.append(time.perf_counter() - t0)
    return port, min(times)


CPU_SAMPLE_FMG = ("one full reconstruction of this workload by the reference's CPU algorithm (serial CIC paint, "
                  "FMG damped Jacobi w=0.4 nu=5, 6 cycles/level, C/OpenMP + scipy.fft); the reference schedule has "
                  "no residual test and stops short of 1e-6")
CPU_SAMPLE_1E6 = ("one full reconstruction of this workload on the host with the GPU's solver (FFT-preconditioned "
                  "defect correction to a 1e-6 relative residual, FP64, C/OpenMP operator + scipy.fft); paint, "
                  "smoothing and read-out as the reference's CPU path")


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    m, bs, bm = workload(args, args.seed)
    port = None
    ts = []
    for i in range(args.warmup + args.steps):
        port, t = cpu_baseline(args, m, bs, bm)
        if i >= args.warmup:
            ts.append(t)
    tm = sum(ts) / len(ts)
    v = 1.0 / tm
    _, t6 = cpu_baseline(args, m, bs, bm, solver="convergent")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tm * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"lightcone MG reconstruction {args.mesh}^3, {args.n_data} data + "
                               f"{args.n_data * args.rand_factor} randoms", "mesh": args.mesh},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": port.threads, "kind": "port", "sample": CPU_SAMPLE_FMG},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "same_config": False,
        "same_config_note": "the reference's CPU path runs its FMG schedule (6 V-cycles per level, no residual "
                            "test); the GPU arm solves to a 1e-6 relative residual. cpu_1e6 times the GPU's solver "
                            "on the host to the same 1e-6 for a like-for-like reading. Box pad 25 Mpc/h instead "
                            "of run!'s hard-coded 500 (cell 5.96 Mpc/h, the workload's stated ~5.9).",
        "cpu_1e6": {"value": 1.0 / t6, "unit": UNIT, "cores": port.threads, "kind": "port", "sample": CPU_SAMPLE_1E6},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_conv_only(args):
    """The network's convolutions alone on a --mesh grid (one JSON line)."""
    import ctypes as C
    import torch
    from baorec import _lib
    cfg = _lib.default_config()
    cfg.method = _lib.MULTIGRID
    for a in range(3):
        cfg.n[a] = args.mesh
        cfg.box_size[a] = 1000.0
    ctx = _lib.Context(cfg)
    torch.cuda.synchronize()
    rows = guess_conv_rooflines(ctx, C, tuple((ci, co, args.mesh) for ci, co, _ in GUESS_CONV_SHAPES))
    print(json.dumps({"metric": "guess convolution TFLOP/s", "mesh": args.mesh, "kernels": rows}), flush=True)
    return 0


def run_stencil_only(args):
    """Finest-level stencil kernels alone (baorec_profile_kernel) on a --mesh
    grid with the lightcone workload's radial line of sight: one JSON line."""
    import ctypes as C
    import torch
    from baorec import _lib
    cfg = _lib.default_config()
    cfg.method = _lib.MULTIGRID
    cfg.mg_mode = _lib.MG_CONVERGENT
    for a, lo in enumerate((500.0, 300.0, 200.0)):
        cfg.n[a] = args.mesh
        cfg.box_size[a] = 2000.0 * args.mesh / 256
        cfg.box_min[a] = lo
    ctx = _lib.Context(cfg)
    torch.cuda.synchronize()
    rows = []
    for spec in filter(None, args.stencil_only.split(",")):
        which, pairs, acc, xy = (list(map(int, spec.split(":"))) + [1, 0, 1])[:4]
        ctx.call("baorec_set_tune_pairs", pairs)
        ctx.call("baorec_set_tune_acc", acc)
        ctx.call("baorec_set_tune_xy", xy)
        avg, nbytes = C.c_float(), C.c_double()
        ctx.call("baorec_profile_kernel", which, args.stencil_reps, C.byref(avg), C.byref(nbytes))
        rows.append({"kernel": which, "pairs": pairs, "acc": acc, "xy": xy, "avg_launch_us": avg.value * 1e3,
                     "algorithmic_GBps": nbytes.value / (avg.value * 1e-3) / 1e9})
    print(json.dumps({"metric": "stencil kernel time", "mesh": args.mesh, "kernels": rows}), flush=True)
    return 0


def run_paint_only(args):
    """The CIC paint of the workload's randoms alone, per mode: one JSON line."""
    import torch
    import baorec
    from baorec import _lib
    m, bs, bm = workload(args, args.seed)
    rec = baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=bs, box_min=bm, los=None,
                                mg_mode="convergent", rtol=1e-6)
    ctx = baorec.setup_fft_(rec, (args.mesh,) * 3)
    R = [torch.from_numpy(a).cuda() for a in (m.rx, m.ry, m.rz, m.rw)]
    nr = int(m.rx.shape[0])
    mesh = torch.zeros(args.mesh ** 3, device="cuda")
    stream = torch.cuda.ExternalStream(ctx.stream)
    torch.cuda.synchronize()
    rows = []
    for mode in filter(None, args.paint_only.split(",")):
        fl = _lib.DETERMINISTIC if mode == "deterministic" else 0
        ctx.call("baorec_set_tune_binned", 1 if mode == "binned" else 0)
        run = lambda f: ctx.call("baorec_cic", mesh.data_ptr(), *[t.data_ptr() for t in R], nr, 0, f)
        run(fl)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.stencil_reps):
            run(fl | _lib.ASYNC)
        e1.record(stream)
        torch.cuda.synchronize()
        rows.append({"mode": mode, "avg_ms": e0.elapsed_time(e1) / args.stencil_reps})
    print(json.dumps({"metric": "paint time", "mesh": args.mesh, "particles": nr, "paints": rows}), flush=True)
    return 0


def run_gb300(args):
    import numpy as np
    import torch
    import ctypes as C
    import baorec
    from baorec import _lib
    if args.conv_only:
        return run_conv_only(args)
    if args.stencil_only:
        return run_stencil_only(args)
    if args.paint_only:
        return run_paint_only(args)

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    m, bs, bm = workload(args, replica_seed(args.seed, rank))
    n = (args.mesh,) * 3
    weights = os.path.join(ROOT, "baorec.jl_gb300", "weights", "guess_lightcone.npy")

    def make(start, gradient="fft"):
        gp = baorec.guess.load_params(weights) if start == "learned" else None
        # the learned start's network runs on the 128^3 restriction of the 256^3 mesh, where it was trained
        rec = baorec.MultigridRecon(bias=2.0, f=0.8, smoothing_radius=15.0, box_size=bs, box_min=bm, los=None,
                                    mg_mode="convergent", rtol=1e-6, nu1=2, nu2=2, max_cycles=50, start=start,
                                    guess_params=gp, gradient=gradient, guess_level=1 if args.mesh == 256 else 0)
        return baorec.setup_fft_(rec, n)

    ctx = make(args.start)
    # the other starts are timed the same way and reported beside the headline,
    # and the headline start with the finite-difference gradient read-out
    others = {} if args.only_start else {s: make(s) for s in ("zero", "spectral", "learned") if s != args.start}
    if not args.only_start:
        others[args.start + "+fd_gradient"] = make(args.start, "fd")
    # launch shapes chosen by the autotuner (per-level stencil tiles, deterministic-paint tile)
    tune = ctx.autotune()
    for c_ in others.values():
        c_.autotune(paint=False)
    setters = {"pair_residual": "baorec_set_tune_pairs", "acc_residual": "baorec_set_tune_acc", "fft_zpass": "baorec_set_tune_zpass",
               "fft_xy_fused": "baorec_set_tune_xy", "stream_residuals": "baorec_set_tune_stream"}
    for kv in filter(None, args.set_tune.split(",")):
        k, v = kv.split("=")
        if k == "tiles":   # per-level tile choices, e.g. tiles=1:1:0:0 (1 = 32x16x16, 0 = 32x8x8)
            bt = [int(x) for x in v.split(":")] + [-1] * 16
            for c_ in [ctx] + list(others.values()):
                c_.call("baorec_set_tune", int(tune["paint_tile"]), (C.c_int32 * 16)(*bt[:16]))
            tune["tile16_per_level"] = bt[:16]
            continue
        for c_ in [ctx] + list(others.values()):
            c_.call(setters[k], int(v))
        tune[k] = int(v)
    nd, nr = len(m.x), len(m.rx)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    X = [dev(a) for a in (m.x, m.y, m.z, m.w)]
    R = [dev(a) for a in (m.rx, m.ry, m.rz, m.rw)]
    out_d = [torch.empty(nd, device="cuda") for _ in range(3)]
    out_rs = [torch.empty(nr, device="cuda") for _ in range(3)]
    out_ri = [torch.empty(nr, device="cuda") for _ in range(3)]
    ptr = lambda ts: [t.data_ptr() for t in ts]
    torch.cuda.synchronize()
    SUM, DISP = _lib.FIELD["sum"], _lib.FIELD["disp"]

    def step(flags=0, xs=None, rs=None, od=None, ors=None, ori=None, ctx=ctx):
        xs = xs or ptr(X)
        rs = rs or ptr(R)
        st = ctx.status("baorec_reconstructed_potential", *xs, nd, *rs, nr, flags)
        if st != _lib.OK:
            _lib.check(ctx.h, st)
        ctx.call("baorec_reconstructed_positions", *xs[:3], nd, SUM, *(od or ptr(out_d)), flags | _lib.ASYNC)
        # the randoms' :sum and :disp positions from one gather of the displacement
        ctx.call("baorec_reconstructed_positions2", *rs[:3], nr, SUM, *(ors or ptr(out_rs)), DISP,
                 *(ori or ptr(out_ri)), flags)

    def timed(c):
        """W warm-up steps, then K steps between CUDA events on the context's stream (max over ranks)."""
        for _ in range(args.warmup):
            step(ctx=c)
        stream = torch.cuda.ExternalStream(c.stream)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        clocks = Clocks(local)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        l0 = c.total_launches()
        clocks.start()
        ev0.record(stream)
        hist = []
        for _ in range(args.steps):
            step(ctx=c)
            s = c.solve_stats()
            hist.append((s["spectral_steps"], s["cycles"]))
        ev1.record(stream)
        torch.cuda.synchronize()
        clk = clocks.stop()
        launches = c.total_launches() - l0
        ms, _ = replica_throughput(ev0.elapsed_time(ev1) / args.steps, ws, dist)
        if dist:
            dist.barrier()
        return ms, hist, clk, launches, c.solve_stats()

    arms = {}
    for s_, c_ in others.items():
        pms, phist, pclk, _, pstats = timed(c_)
        arms[s_] = {"value": ws * 1000.0 / pms, "ms_per_step": pms, "cycles_per_step": [h[1] for h in phist],
                    "spectral_steps_per_step": [h[0] for h in phist],
                    "rel_residual_initial": pstats["rel_residual_initial"],
                    "rel_residual": pstats["rel_residual"], "clocks": pclk}
    ms, hist, clk, launches, stats = timed(ctx)
    cycles = [h[1] for h in hist]
    value = ws * 1000.0 / ms

    # rooflines measured live (CUDA events on the context stream around a run
    # of launches on the finest level); the headline is the dominant kernel of
    # the timed path: the largest device time per reconstruction (launches per
    # reconstruction of the last timed solve x the live per-launch time) among
    # the FP32 running residual of the FFT corrections, the accurate residual
    # and the batched xy transforms for the FFT / learned starts; the
    # red-black sweep for the plain multigrid start
    peak, peak_src = measured_peak()
    N = int(np.prod(n))
    xy_fused = bool(tune.get("fft_xy_fused", 0))
    names = {0: "rb_sweep2_kernel", 1: "resid_acc2_kernel", 3: RUNNING_RESIDUAL[tune.get("pair_residual", 0)],
             4: "resid_acc_stream_kernel", 5: "resid_diff_stream_kernel",
             8: ("xy_r2c_kernel (fused xy forward transform, four-CTA clusters)" if xy_fused
                 else "cuFFT xy forward transform (two passes)"),
             9: ("xy_c2r_kernel (fused xy inverse transform, four-CTA clusters)" if xy_fused
                 else "cuFFT xy inverse transform (two passes)")}
    meas = {}
    kinds = (0, 1, 3, 4, 5) + ((8, 9) if n[2] == 256 and tune.get("fft_zpass", 0) else ())
    for which in (() if args.no_kernels else kinds):
        avg, nbytes = C.c_float(), C.c_double()
        ctx.call("baorec_profile_kernel", which, 30, C.byref(avg), C.byref(nbytes))
        ach = nbytes.value / (avg.value * 1e-3) / 1e9
        meas[which] = {"kernel": names[which], "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                       "frac": ach / peak, "peak_source": peak_src,
                       "traffic": traffic_per_launch(names[which].split()[0], N),
                       "algorithmic_bytes_per_launch": nbytes.value, "avg_launch_ms": avg.value}
    # every form of the FP32 running residual (tune.pairs 0-6), timed the same way; the tuner's choice restored
    if meas:
        forms = {}
        chosen = ctx.lib.baorec_tune_pairs(ctx.h)
        for form in range(7):
            ctx.call("baorec_set_tune_pairs", form)
            avg, nbytes = C.c_float(), C.c_double()
            ctx.call("baorec_profile_kernel", 3, 30, C.byref(avg), C.byref(nbytes))
            forms["%d: %s" % (form, RUNNING_RESIDUAL[form])] = {
                "avg_launch_ms": avg.value, "frac": nbytes.value / (avg.value * 1e-3) / 1e9 / peak}
        ctx.call("baorec_set_tune_pairs", chosen)
        meas["pair_forms"] = forms
        # the batched xy transforms of the FFT corrections: cuFFT's two passes
        # against the fused cluster kernels, the tuner's choice restored
        if n[2] == 256:
            xyf = {}
            chosen = ctx.lib.baorec_tune_xy(ctx.h)
            for xy, label in ((0, "cuFFT"), (1, "fused cluster kernels")):
                ctx.call("baorec_set_tune_xy", xy)
                for which, d in ((8, "forward"), (9, "inverse")):
                    avg, nbytes = C.c_float(), C.c_double()
                    ctx.call("baorec_profile_kernel", which, 30, C.byref(avg), C.byref(nbytes))
                    xyf["%s %s" % (label, d)] = {
                        "avg_launch_ms": avg.value, "algorithmic_bytes_per_launch": nbytes.value,
                        "frac": nbytes.value / (avg.value * 1e-3) / 1e9 / peak}
            ctx.call("baorec_set_tune_xy", chosen)
            xyf["chosen"] = "fused cluster kernels" if chosen else "cuFFT"
            meas["xy_transforms"] = xyf
    # V-cycles/s: one V-cycle of the residual-driven solve (the plain start's
    # step) and one of the reference's schedule (vcycle!), on the finest level
    vcycles = {}
    for which, label in (() if args.no_kernels else ((6, "residual-driven (red-black 2+2, every level)"),
                                                     (7, "reference vcycle! (damped Jacobi 5+5, every level)"))):
        avg, nbytes = C.c_float(), C.c_double()
        ctx.call("baorec_profile_kernel", which, 10, C.byref(avg), C.byref(nbytes))
        vcycles[label] = {"per_s": 1000.0 / avg.value, "ms": avg.value, "algorithmic_bytes": nbytes.value,
                          "achieved": nbytes.value / (avg.value * 1e-3) / 1e9, "unit": "GB/s", "peak": peak,
                          "frac": nbytes.value / (avg.value * 1e-3) / 1e9 / peak}
    head = 0 if args.start == "zero" else (5 if tune.get("stream_residuals", -1) != 0 else 3)
    device_ms = {}
    if meas and args.start != "zero":
        corr = int(stats["spectral_steps"])
        n_acc = max(len(ctx.solve_history()) - 1, 0)   # one accurate residual after each outer step
        units = {head: max(corr - n_acc, 0), 1: n_acc}
        if 8 in meas:   # the corrections, the smoothing pair (two meshes) and the displacement (1 / 3 meshes)
            units[8], units[9] = corr + 3, corr + 5
        device_ms = {w: u * meas[w]["avg_launch_ms"] for w, u in units.items()}
        head = max(device_ms, key=device_ms.get)
    roofline, aux = None, {}
    if meas:
        roofline = dict(meas[head])
        roofline["kernel"] = "%s (finest level %s)" % (names[head], "x".join(map(str, n)))
        if device_ms:
            roofline["device_ms_per_reconstruction"] = {names[w].split()[0] if w not in (8, 9) else names[w]: v
                                                        for w, v in device_ms.items()}
        aux = {names[w]: meas[w] for w in meas if w != head and w not in ("pair_forms", "xy_transforms")}
        if "pair_forms" in meas:
            aux["running residual forms"] = meas["pair_forms"]
        if "xy_transforms" in meas:
            aux["xy transforms"] = meas["xy_transforms"]

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        hX = [pin(a) for a in (m.x, m.y, m.z, m.w)]
        hR = [pin(a) for a in (m.rx, m.ry, m.rz, m.rw)]
        hod = [torch.empty(nd).pin_memory() for _ in range(3)]
        hors = [torch.empty(nr).pin_memory() for _ in range(3)]
        hori = [torch.empty(nr).pin_memory() for _ in range(3)]
        hp = lambda ts: [t.data_ptr() for t in ts]
        kw = dict(xs=hp(hX), rs=hp(hR), od=hp(hod), ors=hp(hors), ori=hp(hori))
        step(_lib.HOST, **kw)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step(_lib.HOST, **kw)
        torch.cuda.synchronize()
        te = (time.perf_counter() - t0) / args.steps
        e2e = {"value": ws / te, "unit": UNIT,
               # potential: x,y,z,w of both catalogs; each read-out call stages x,y,z again
               "h2d_bytes_per_step": 16 * (nd + nr) + 12 * nd + 12 * nr,
               "d2h_bytes_per_step": 12 * nd + 24 * nr, "ms_per_step": te * 1e3}

    # particles painted/s: the 5e6 randoms into a 256^3 mesh, float-atomic, binned and deterministic paints
    stream = torch.cuda.ExternalStream(ctx.stream)
    scratch = torch.zeros(N, device="cuda")
    binned = ctx.lib.baorec_tune_binned(ctx.h)
    for label, fl, mode in (() if args.no_kernels else
                            (("cic_paint (atomic)", 0, 0),
                             ("cic_paint (binned: tile sort + shared-memory tiles)", 0, 1),
                             ("cic_paint (deterministic, tile sort)", _lib.DETERMINISTIC, binned))):
        ctx.call("baorec_set_tune_binned", mode)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 10
        ctx.call("baorec_cic", scratch.data_ptr(), *ptr(R), nr, 0, fl)
        e0.record(stream)
        for _ in range(reps):
            ctx.call("baorec_cic", scratch.data_ptr(), *ptr(R), nr, 0, fl | _lib.ASYNC)
        e1.record(stream)
        torch.cuda.synchronize()
        pms = e0.elapsed_time(e1) / reps
        pbytes = 16.0 * nr + 4.0 * N
        aux[label] = {"particles_per_s": nr * 1e3 / pms, "avg_launch_ms": pms, "algorithmic_bytes": pbytes,
                      "achieved": pbytes / (pms * 1e-3) / 1e9, "unit": "GB/s", "peak": peak,
                      "frac": pbytes / (pms * 1e-3) / 1e9 / peak}
    ctx.call("baorec_set_tune_binned", binned)
    del scratch

    if not args.no_kernels and args.mesh % 128 == 0:
        aux.update(guess_conv_rooflines(ctx, C))
    if not args.no_kernels:
        aux["power multipoles (survey, l = 0, 2, 4)"] = power_timing(args, baorec, torch, np, X, R, bs, bm)

    batch = None if args.no_batch else run_batch(args, torch, np)
    box, box_state = run_box(args, torch, np)
    scale = None
    if args.scale512 and args.mesh == 256:
        try:
            scale = run_scale_512(args, torch, np, checks=(rank == 0 and ws == 1 and not args.no_cpu))
        except Exception as exc:   # the headline line is printed whatever happens here
            scale = {"error": f"{type(exc).__name__}: {exc}"}
        torch.cuda.empty_cache()

    # the metric's own comparison: learned-start recons/s over plain-multigrid recons/s
    rates = {args.start: value}
    rates.update({k: v["value"] for k, v in arms.items()})
    learned_vs_plain = rates["learned"] / rates["zero"] if "learned" in rates and "zero" in rates else None
    spectral_vs_plain = rates["spectral"] / rates["zero"] if "spectral" in rates and "zero" in rates else None

    cpu, checks = None, None
    if rank == 0 and ws == 1 and not args.no_cpu:
        port, tc = cpu_baseline(args, m, bs, bm)
        _, t6 = cpu_baseline(args, m, bs, bm, solver="convergent")
        cpu = {"value": 1.0 / tc, "unit": UNIT, "cores": port.threads, "kind": "port", "sample": CPU_SAMPLE_FMG,
               "same_config": False,
               "cpu_1e6": {"value": 1.0 / t6, "unit": UNIT, "cores": port.threads, "kind": "port",
                           "sample": CPU_SAMPLE_1E6}}
        solvers = {args.start: ctx}
        solvers.update({k: v for k, v in others.items() if "+" not in k})
        checks = oracle_checks(args, torch, np, solvers, m, bs, bm, X, R, box_state)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"lightcone MG reconstruction {args.mesh}^3 to 1e-6 relative residual, "
                                   f"{nd} data + {nr} randoms, CIC, R=15, b=2, f=0.8, local LOS, 2+2 RB sweeps",
                       "mesh": args.mesh, "start": args.start, "autotune": tune,
                       "fft_callback": ctx.fft_callbacks(),
                       "l2": "working set per step > 1 GB >> 126 MB L2 (inputs larger than L2)",
                       "parallelism": f"replicas x{ws}"},
            "solver": {"start": args.start, "cycles": stats["cycles"], "spectral_steps": stats["spectral_steps"],
                       "rel_residual": stats["rel_residual"], "cycles_per_step": cycles,
                       "spectral_steps_per_step": [h[0] for h in hist]},
            "starts": arms,
            "learned_vs_plain": learned_vs_plain,
            "spectral_vs_plain": spectral_vs_plain,
            "l2_vs_fp64": None if checks is None else {
                "lightcone_%d" % args.mesh: checks["lightcone_%d" % args.mesh]["solve"][args.start]["l2"],
                "box_128": checks["box_128"]["l2"]},
            "accuracy": checks,
            "box": box,
            "scale_512": scale,
            "gpu_launches": launches,
            "clocks": clk,
            "roofline": roofline,
            "kernels": aux,
            "vcycles": vcycles,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "batch": batch,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
