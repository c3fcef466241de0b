"""Benchmark: 256^3 pressure-Poisson time-to-1e-8 on one GB300.

One step = one complete solve of the C3 workload (256^3 cells, periodic x/y,
Neumann z, 1000 masked spheres of radius 6 cells, spectral RHS) to a true
relative residual of 1e-8, inputs resident in HBM.  The headline method is the
fastest available form (learned guess + FP32-inner/FP64-refined PCG when a
trained network is given, else FP32-inner/FP64-refined PCG); plain FP64 PCG is
timed beside it.  The metric is solves/s (higher is better).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU form (the plain-C FP64
oracle, OpenMP on all host cores) on a bounded sample of the same workload.
"""
import argparse
import faulthandler
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "bluebottle-3.0_gb300"))

METRIC = "256³ Poisson time-to-1e-8 residual: learned+mixed vs plain FP64 PCG, one GB300"
UNIT = "solves/s"
WORKLOAD = ("C3: 256^3 cells, periodic x/y + Neumann z, 1000 spheres r=6 cells, k^-11/3 RHS (step 1 of an OU "
            "sequence), tol 1e-8 (true rel.)")
# DRAM bytes (read + write) per launch of the dominant kernels on this workload,
# from one ncu capture each (--set full, two launches of a 256^3 solve; the
# summaries sit with the other profiles): kernel kind -> bytes
NCU_TRAFFIC = {"search_spmv_f32": 226.697984e6 + 150.230784e6, "search_spmv": 432.974336e6 + 360.291072e6,
               "update_f32": 134.251008e6 + 20.922112e6, "update": 268.485376e6 + 92.526592e6,
               "fused_f32": 307.027712e6 + 216.193536e6}


# FP64-pipe thread instructions per cell per launch of the plain FP64 kernels on
# this workload (interior neighbour sums on the integer pipe), from one ncu
# capture of sm__thread_inst_executed_pipe_fp64_pred_on (the summary sits with
# the other profiles): kernel kind -> instructions per cell
NCU_FP64_INST = {"search_spmv": 72.429664e6 / 16777216, "update": 38.618304e6 / 16777216}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "fallback": True}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit())
        smax = max((float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()), default=None)
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for nm, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def dist_init(n, select_device=True):
    """One process per GPU under torchrun; replicas only (no collective on the
    data path).  Each rank solves on GPU LOCAL_RANK; the host-side gloo group
    carries only the barrier and the max over ranks of the step time.
    Returns (rank, world, barrier, max_reduce)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world <= 1:
        return 0, 1, (lambda: None), (lambda v: v)
    if select_device:
        import bbpp
        bbpp._check(bbpp.lib().bbpp_set_device(int(os.environ.get("LOCAL_RANK", "0"))))
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo")

    def barrier():
        dist.barrier()

    def vmax(v):
        t = torch.tensor([float(v)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return rank, world, barrier, vmax


def aggregate(world, ms_max):
    """Whole-job solves/s of `world` replicas whose slowest step took ms_max."""
    return world * 1000.0 / ms_max


def make_c3():
    import numpy as np
    import bbpp
    from bbpp import problems
    c = problems.CONFIGS["C3"]
    g = problems.make_grid(c["n"], c["bc"])
    cents, radii = problems.place_spheres(g, c["nsph"], c["rad"], c["seed"])
    return g, cents, radii, c


def train_c4_net(args):
    """The learned guess per the C4 workload: OU triples at 64^3 (128 spheres of
    radius 4 cells), p* by plain FP64 PCG to 1e-10, Adam on the GPU.  A saved
    network (--net) skips the training."""
    from bbpp import learned, problems
    net = learned.Net(seed=1)
    info = {}
    if args.net and os.path.exists(args.net):
        net.load(args.net)
        info["loaded"] = args.net
        return net, info
    c = problems.CONFIGS["C4"]
    t0 = time.time()
    data, g4, _ = learned.make_ou_dataset(c["n"], args.train_samples, nsph=c["nsph"], rad=c["rad"], seed=c["seed"],
                                          tol=c["tol"])
    t1 = time.time()
    hist = net.train(data, steps=args.train_steps, batch=4, lr=2e-3)
    import numpy as np
    info = {"samples": args.train_samples, "steps": args.train_steps, "data_s": round(t1 - t0, 1),
            "train_s": round(time.time() - t1, 1), "loss_first": float(np.mean(hist[:10])),
            "loss_last": float(np.mean(hist[-50:]))}
    if args.net:
        net.save(args.net)
    return net, info


def reference_gpu(g, mask, rhs, tol, args):
    """The reference's own CUDA solve (its kernels from oracle/_ref/ref_solver.cubin
    under the restated one-rank host loop of src/cuda_solver.cu) on the same
    workload and GPU, with its own stopping rule (r,z) <= tol^2 (b,b)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle", "refgpu"))
    try:
        import pyrefgpu
    except Exception as e:  # noqa: BLE001
        return {"unavailable": "harness import failed: %s" % e}
    if not pyrefgpu.available():
        return {"unavailable": "reference cubin not built (needs the reference tree at build time)"}
    bc = tuple(int(v) for v in g.bc)
    ref = pyrefgpu.RefSolver(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, bc, mask)
    times, its = [], []
    for i in range(2):
        phi, it, res, ms, rc = ref.solve(rhs, tol)
        if rc != 0:
            ref.close()
            return {"unavailable": "reference solve status %d" % rc}
        times.append(ms)
        its.append(it)
    # the same solver run tight (pp_residual 2e-15: a true relative residual
    # near 1e-12 at this size), the FP64 solution the methods are also compared with
    phi, it_t, res_t, ms_t, rc_t = ref.solve(rhs, 2e-15)
    ref.close()
    ms = float(np.mean(times[1:]))
    out = {"value": 1000.0 / ms, "unit": UNIT, "ms_per_solve": ms, "iters": its[-1],
           "stop": "(r,z) <= tol^2 (b,b), the reference's rule",
           "kind": "reference CUDA kernels (src/solver_kernel.cu, unmodified) on this GPU, one rank"}
    if rc_t == 0:
        out["tight"] = {"pp_residual": 2e-15, "iters": it_t}
        out["_phi"] = phi
    return out


def profiler_api():
    """cuProfilerStart/Stop of the driver for the current context (a no-op
    where the driver library is missing)."""
    import ctypes
    try:
        cu = ctypes.CDLL("libcuda.so.1")
    except OSError:
        return lambda on: None
    return lambda on: (cu.cuProfilerStart() if on else cu.cuProfilerStop())


def cpu_model():
    """The host CPU's model name (lscpu), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:  # noqa: BLE001
        pass
    import platform
    return platform.processor() or platform.machine()


def oracle_mod():
    """The CPU oracle (pyoracle) and its input generator (pyproblems)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    import pyproblems
    return pyoracle, pyproblems


def oracle_solve(og, rhs, mask, tol, x0=None):
    """One complete plain FP64 Jacobi-PCG solve by the oracle (OpenMP over the
    host cores) to a true relative residual of tol: (seconds, x, result)."""
    pyoracle, _ = oracle_mod()
    t0 = time.perf_counter()
    x, res = pyoracle.pcg(og, rhs, mask, tol=tol, x0=x0)
    t = time.perf_counter() - t0
    if res["status"] != 0:
        raise RuntimeError("oracle solve did not converge: %s" % res)
    return t, x, res


def pyoracle_true_rel(g, rhs, x, mask):
    """||rhs - (-A)x|| / ||rhs|| by the oracle."""
    pyoracle, _ = oracle_mod()
    return float(pyoracle.true_rel(pyoracle.from_tuple(g.as_tuple()), rhs, x, mask))


def run_reference(args):
    """CPU arm: the reference's algorithm in plain C (the oracle, OpenMP on all
    host cores).  Every step is one complete solve of the C3 workload to the
    same 1e-8 true relative residual; the inputs come from the oracle's own
    generator, so this arm loads no library of the solver."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)  # before the oracle's OpenMP runtime starts
    import numpy as np
    pyoracle, pyproblems = oracle_mod()
    og, mask, cents, radii, seed, tol = pyproblems.workload("C3")
    seq = pyproblems.OUFields((og.nz, og.ny, og.nx), seed, mask)
    seq.current()
    rhs = seq.advance()  # step 1 of the OU sequence: the GPU arm's right-hand side
    times, iters = [], None
    for s in range(args.warmup + args.steps):
        t, x, res = oracle_solve(og, rhs, mask, tol)
        if s >= args.warmup:
            times.append(t)
            iters = res["iters"]
    sec = float(np.mean(times))
    value = 1.0 / sec
    sample = ("each step one complete oracle PCG solve of the C3 workload (256^3, 1000 spheres) from zero to a "
              "1e-8 true relative residual: %d iterations, %.2f s mean over %d steps" % (iters, sec, len(times)))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sec * 1000.0, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "method": "plain FP64 Jacobi PCG (oracle port, OpenMP)"},
            "iters": iters,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "cpu": cpu_model(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args):
    import numpy as np
    import bbpp
    from bbpp import problems
    rank, world, barrier, vmax = dist_init(args.gpus)
    g, cents, radii, c = make_c3()
    s = bbpp.Solver(g)
    dmask = bbpp.DeviceArray(g.shape, np.uint8)
    s.sphere_mask(cents, radii, dmask)
    mask = dmask.download()
    # the solve at step t of an OU sequence on the C3 geometry; step t-1 gives
    # the previous pressure the learned guess starts from
    seq = problems.OUSequence(g.shape, c["seed"], mask)
    rhs_prev = seq.field()
    rhs = seq.step()
    drhs = bbpp.DeviceArray.from_host(rhs_prev)
    dprev = bbpp.DeviceArray(g.shape, np.float64)
    s.solve(drhs, dprev, dmask, tol=1e-10, precision=bbpp.FP64)
    drhs.upload(rhs)
    dx = bbpp.DeviceArray(g.shape, np.float64)
    N = g.n
    tol = c["tol"]

    net = None
    net_info = None
    methods = {"fp64": dict(precision=bbpp.FP64), "ir": dict(precision=bbpp.FP32_IR),
               "ir_restart": dict(precision=bbpp.FP32_IR, ir_mode=bbpp.IR_RESTART),
               "ir_every50": dict(precision=bbpp.FP32_IR, ir_drop=0.0),
               "ir_warm": dict(precision=bbpp.FP32_IR, guess=bbpp.GUESS_GIVEN)}
    headline = "ir"
    if not args.no_learned and args.only in (None, "learned_ir", "learned_ir_fine"):
        net, net_info = train_c4_net(args)
        methods["learned_ir"] = dict(precision=bbpp.FP32_IR, guess=bbpp.GUESS_LEARNED, net=net.handle,
                                     prev=dprev.ptr)
        # the same network run on the 256^3 grid itself instead of the grid restricted by 2
        methods["learned_ir_fine"] = dict(precision=bbpp.FP32_IR, guess=bbpp.GUESS_LEARNED, net=net.handle,
                                          prev=dprev.ptr, net_coarsen=1)
        headline = "learned_ir"

    def step(kw):
        if kw.get("guess") == bbpp.GUESS_GIVEN:
            dx.upload(prev_host)  # warm start: x = p_prev before the (timed) solve
        bbpp.flush_l2()
        return s.solve(drhs, dx, dmask, tol=tol, **kw)

    prev_host = dprev.download()

    if args.only:
        # solves of one method only (profiler runs): steps solves, no warm-up;
        # the profiler's collection is switched on around them only
        # (ncu --profile-from-start off)
        prof = profiler_api()
        prof(True)
        for _ in range(args.steps):
            rep = step(methods[args.only])
            assert rep.status == bbpp.CONVERGED
        bbpp.sync()
        prof(False)
        print(json.dumps({"only": args.only, "iters": rep.iters, "ms": rep.ms, "guess_ms": rep.guess_ms,
                          "launches": rep.launches}))
        return

    for name, kw in methods.items():
        for _ in range(args.warmup):
            rep = step(kw)
            assert rep.status == bbpp.CONVERGED, (name, rep.as_dict())

    # The FP64 solution each method is measured against: the CPU oracle's plain
    # FP64 PCG, from zero to a 1e-8 true relative residual (timed: that solve is
    # the CPU baseline), then continued from there to 1e-12.  With --no-cpu it is
    # this library's plain FP64 PCG to 1e-12 instead (the tests pin that solver to
    # the oracle).
    cpu = None
    ref_kind = "library FP64 PCG to a 1e-12 true relative residual"
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        pyoracle, _ = oracle_mod()
        og = pyoracle.from_tuple(g.as_tuple())
        t_cpu, x_cpu, r_cpu = oracle_solve(og, rhs, mask, tol)
        _, xref, r_tight = oracle_solve(og, rhs, mask, 1e-12, x0=x_cpu)
        cpu = {"value": 1.0 / t_cpu, "unit": UNIT, "cores": threads, "cpu": cpu_model(), "kind": "port",
               "sample": "one complete oracle PCG solve of this workload from zero to a 1e-8 true relative "
                         "residual (%d iterations, %.2f s, OpenMP on all host cores)" % (r_cpu["iters"], t_cpu)}
        ref_kind = "CPU oracle FP64 PCG to a %.1e true relative residual" % r_tight["true_rel"]
    else:
        dref = bbpp.DeviceArray(g.shape, np.float64)
        rref = s.solve(drhs, dref, dmask, tol=1e-12, precision=bbpp.FP64)
        assert rref.status == bbpp.CONVERGED
        xref = dref.download()
        del dref
    xref_max = float(np.abs(xref).max())

    res = {}
    xkeep = {}
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    for name, kw in methods.items():
        reps = []
        barrier()
        bbpp.sync()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            reps.append(step(kw))
        bbpp.sync()
        wall = time.perf_counter() - t0
        barrier()
        ms = float(np.mean([r.ms for r in reps]))
        ms = vmax(ms)
        # max error of the last solve's x against the FP64 solution (outside the timed loop)
        xlast = dx.download()
        err = float(np.abs(xlast - xref).max()) / xref_max
        if name in ("fp64", headline):
            xkeep[name] = xlast
        res[name] = dict(ms=ms, guess_ms=float(np.mean([r.guess_ms for r in reps])), iters=reps[-1].iters,
                         outer=reps[-1].outer, true_rel=reps[-1].true_rel,
                         max_err_vs_fp64=err, bytes=reps[-1].bytes, launches=int(sum(r.launches for r in reps)),
                         wall_s=wall, status=[r.status for r in reps], all_ms=[r.ms for r in reps])
    clk = clocks.stop()
    # per-kernel device time: the same solves again with CUDA events around
    # every kernel on the solver stream (direct launches instead of graphs)
    for name, kw in methods.items():
        s.set_profiling(True)
        for _ in range(max(1, min(args.steps, 2))):
            step(kw)
        res[name]["kstats"] = s.kernel_stats()
        s.set_profiling(False)

    # end to end: host (pinned) buffers in, solution out, copies inside the timed call
    hr = bbpp.PinnedArray(g.shape, np.float64)
    hm = bbpp.PinnedArray(g.shape, np.uint8)
    hx = bbpp.PinnedArray(g.shape, np.float64)
    hr.array[...] = rhs
    hm.array[...] = mask
    e2e_t = []
    o = bbpp.default_opts(tol=tol, **methods[headline])
    hp = bbpp.PinnedArray(g.shape, np.float64)
    hp.array[...] = prev_host
    import ctypes
    for i in range(args.warmup + args.steps):
        rep = bbpp.Report()
        bbpp.flush_l2()
        t0 = time.perf_counter()
        # the previous pressure also comes from the host (pinned) for the learned guess
        if headline == "learned_ir":
            bbpp.lib().bbpp_h2d(dprev.ptr, hp.ptr, N * 8)
        rc = bbpp.lib().bbpp_solve_host(s.handle, hm.ptr, hr.ptr, hx.ptr, ctypes.byref(o), ctypes.byref(rep))
        t1 = time.perf_counter()
        assert rc == bbpp.CONVERGED, rc
        if i >= args.warmup:
            e2e_t.append(t1 - t0)
    e2e_v = world / vmax(float(np.mean(e2e_t)))
    xh = hx.array.copy()

    # roofline of the dominant kernel of the headline method
    pk = peaks()
    hb = pk.get("hbm_gbs", 6800.0)

    def roof(name):
        ks = res[name]["kstats"]
        if not ks:
            return None
        top = max(ks, key=lambda k: k[2])
        kname, nl, kms, kbytes = top
        achieved = (kbytes / nl) / (kms / nl * 1e-3) / 1e9
        tot = sum(k[2] for k in ks)
        out = {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": hb, "unit": "GB/s",
               "frac": achieved / hb, "traffic": NCU_TRAFFIC.get(kname), "algorithmic_bytes": kbytes / nl,
               "launches": nl, "avg_us": kms / nl * 1e3,
               "share": kms / tot if tot else None,
               "peak_source": "measured" if "fallback" not in pk else "fallback"}
        if kname == "fused_f32" and stream_gbs:
            # what a plain streaming kernel with the same per-cell traffic reaches on this GPU
            out["stream_same_mix_gbs"] = stream_gbs
            out["frac_of_stream_same_mix"] = achieved / stream_gbs
        return out

    def fp64_roof(name):
        """The plain FP64 solve against the FP64 pipe (1/64 of the FP32 rate on
        this part; its update kernel is bound by it): FP64 thread instructions
        of its kernels (per cell, from ncu) over their CUDA-event time, against
        the FMA rate this GPU issues (bbpp_fp64_fma_rate)."""
        ks = res[name]["kstats"]
        if not ks or not fma_rate:
            return None
        inst, ms = 0.0, 0.0
        for kname, nl, kms, _ in ks:
            if kname in NCU_FP64_INST:
                inst += NCU_FP64_INST[kname] * N * nl
                ms += kms
        if ms == 0.0:
            return {"peak_fma_per_s": fma_rate, "unit": "FP64 inst/s"}
        achieved = inst / (ms * 1e-3)
        return {"resource": "fp64 pipe", "achieved": achieved, "peak": fma_rate, "unit": "FP64 inst/s",
                "frac": achieved / fma_rate, "inst_per_cell": {k: v for k, v in NCU_FP64_INST.items()},
                "kernels_ms_share": ms / sum(k[2] for k in ks), "peak_source": "bbpp_fp64_fma_rate (this run)"}

    fma_rate = stream_gbs = None
    try:
        fma_rate = bbpp.fp64_fma_rate()
        stream_gbs = bbpp.stream_mix_rate(N) / 1e9
    except Exception:  # noqa: BLE001
        pass
    H = res[headline]
    value = aggregate(world, H["ms"])
    plain = res["fp64"]

    ref_gpu = reference_gpu(g, mask, rhs, tol, args) if rank == 0 and not args.no_cpu else None
    if ref_gpu is not None and "ms_per_solve" in ref_gpu:
        # this library's plain FP64 PCG under the reference's stopping rule: the same work
        reps = []
        for _ in range(3):
            reps.append(step(dict(precision=bbpp.FP64, stop=bbpp.STOP_REF_RZ)))
        ref_gpu["ours_fp64_same_rule"] = {"ms_per_solve": float(np.mean([r.ms for r in reps[1:]])),
                                          "iters": reps[-1].iters}
        ref_gpu["speedup_fp64_same_rule"] = ref_gpu["ms_per_solve"] / ref_gpu["ours_fp64_same_rule"]["ms_per_solve"]
    if ref_gpu is not None and "_phi" in ref_gpu:
        phi = ref_gpu.pop("_phi")
        pmax = float(np.abs(phi).max())
        ref_gpu["tight"]["true_rel"] = pyoracle_true_rel(g, rhs, phi, mask)
        # max |x - x_ref| / max |x_ref| of the last timed solve of each method
        ref_gpu["tight"]["max_err"] = {k: float(np.abs(v - phi).max()) / pmax for k, v in xkeep.items()}
        ref_gpu["tight"]["oracle_vs_reference_max_err"] = float(np.abs(xref - phi).max()) / pmax

    def canon_gbs(r):
        return r["bytes"] / (r["ms"] * 1e-3) / 1e9

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": H["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        # arithmetic of the headline method: FP32 PCG vectors with FP64 residuals, solution and dot
        # accumulators (plus the BF16 network of the learned guess)
        "dtype": {"ir": "f32-inner/f64-refined", "learned_ir": "f32-inner/f64-refined (+bf16 guess)"}.get(headline,
                                                                                                       "f64"),
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "method": {"ir": "FP32 Jacobi PCG with FP64 reliable updates",
                                                     "learned_ir": "learned guess (C4 net, run on the grid "
                                                                   "restricted by 2) + FP32 Jacobi PCG with "
                                                                   "FP64 reliable updates",
                                                     "fp64": "plain FP64 Jacobi PCG"}[headline],
                   "l2": "flushed (512 MB write) before every step; working set 0.9 GB > L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "iters": H["iters"], "outer": H["outer"], "true_rel": H["true_rel"],
        # max |x - x64| / max |x64|, x64 the FP64 solution named by max_err_reference
        "max_err_vs_fp64": H["max_err_vs_fp64"], "max_err_reference": ref_kind,
        "plain_fp64": {"value": aggregate(world, plain["ms"]), "ms_per_step": plain["ms"], "iters": plain["iters"],
                       "true_rel": plain["true_rel"], "max_err_vs_fp64": plain["max_err_vs_fp64"],
                       "canonical_gbs": canon_gbs(plain),
                       "canonical_frac": canon_gbs(plain) / hb, "roofline": roof("fp64"),
                       "fp64_roofline": fp64_roof("fp64")},
        "speedup_vs_plain_fp64": plain["ms"] / H["ms"],
        "canonical_gbs": canon_gbs(H),
        "roofline": roof(headline),
        "e2e": {"value": e2e_v, "unit": UNIT,
                "h2d_bytes_per_step": int(N * 9 + (N * 8 if headline == "learned_ir" else 0)),
                "d2h_bytes_per_step": int(N * 8)},
        "methods": {k: {"ms": v["ms"], "guess_ms": v["guess_ms"], "iters": v["iters"], "outer": v["outer"],
                        "true_rel": v["true_rel"], "max_err_vs_fp64": v["max_err_vs_fp64"],
                        "solves_per_s": 1000.0 / v["ms"]}
                    for k, v in res.items()},
        "learned_training": net_info,
        "gpu_launches": H["launches"],
        "clocks": clk,
        "cpu_baseline": cpu,
        "reference_gpu": ref_gpu,
    }
    if rank == 0:
        print(json.dumps(line))


C5_METRIC = ("512³ OU sequence (50 solves) time-to-1e-8 residual: learned+mixed vs warm-started plain FP64 PCG, "
             "one GB300")
C5_WORKLOAD = ("C5: 512^3 cells, periodic x/y + Neumann z, 4000 spheres r=5 cells (fixed layout), OU-evolved "
               "k^-11/3 RHS (correlation 0.95 per step), consecutive solves to tol 1e-8 (true rel.)")


def run_c5(args):
    """The combined form at scale: consecutive solves of an OU-evolved sequence
    on the 512^3 geometry, as the reference's time loop calls its pressure solve
    once per inner iteration.  Every solve of the headline method starts from
    the learned guess on the previous pressure and runs FP32 PCG with FP64
    reliable updates to 1e-8; the baseline is plain FP64 PCG warm-started from
    its previous solution; FP32/FP64 PCG warm-started from the previous pressure
    (no network) shows what the network adds.  Each method runs its own
    sequence from the same first pressure.  One JSON line."""
    import numpy as np
    import torch
    import bbpp
    from bbpp import problems
    rank, world, barrier, vmax = dist_init(args.gpus)
    c = problems.CONFIGS["C5"]
    nsolves = args.c5_solves
    g = problems.make_grid(c["n"], c["bc"])
    t0 = time.time()
    cents, radii = problems.place_spheres(g, c["nsph"], c["rad"], c["seed"])
    s = bbpp.Solver(g)
    dmask = bbpp.DeviceArray(g.shape, np.uint8)
    s.sphere_mask(cents, radii, dmask)
    mask = dmask.download()
    net, net_info = train_c4_net(args)
    setup_s = time.time() - t0
    tol = c["tol"]
    dev = torch.device("cuda")
    seq = problems.OUSequenceDevice(g.shape, c["seed"], mask, device="cuda")
    rhs = seq.field()
    torch.cuda.synchronize()
    p0 = torch.zeros(g.shape, dtype=torch.float64, device=dev)
    dv = bbpp.DeviceView.of_tensor  # the solver reads the torch tensors in place
    rep0 = s.solve(dv(rhs), dv(p0), dmask, tol=tol, precision=bbpp.FP64)
    assert rep0.status == bbpp.CONVERGED
    methods = {
        "learned_ir": dict(precision=bbpp.FP32_IR, guess=bbpp.GUESS_LEARNED, net=net.handle),
        "fp64_warm": dict(precision=bbpp.FP64, guess=bbpp.GUESS_GIVEN),
        "ir_warm": dict(precision=bbpp.FP32_IR, guess=bbpp.GUESS_GIVEN),
    }
    # per method: the previous solution and the output buffer (the learned
    # guess reads prev and writes x, so they are two buffers, swapped per step)
    state = {k: [p0.clone(), torch.empty_like(p0)] for k in methods}
    rec = {k: [] for k in methods}
    tight_every = max(1, nsolves // 5)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    for t in range(1, nsolves + 1):
        rhs = seq.step()
        torch.cuda.synchronize()
        xs = {}
        for name, kw in methods.items():
            prev, out = state[name]
            if kw["guess"] == bbpp.GUESS_GIVEN:
                out.copy_(prev)
                torch.cuda.synchronize()
                rep = s.solve(dv(rhs), dv(out), dmask, tol=tol, **kw)
            else:
                rep = s.solve(dv(rhs), dv(out), dmask, tol=tol, prev=prev.data_ptr(), **kw)
            assert rep.status == bbpp.CONVERGED, (name, t, rep.as_dict())
            rec[name].append({"ms": rep.ms, "guess_ms": rep.guess_ms, "iters": rep.iters, "true_rel": rep.true_rel,
                              "launches": rep.launches})
            state[name] = [out, prev]
            xs[name] = out
        # max |x - x_fp64| / max |x_fp64| against the warm-started FP64 solve of the same step
        base = xs["fp64_warm"]
        bmax = float(base.abs().max())
        for name in methods:
            rec[name][-1]["max_err_vs_fp64"] = float((xs[name] - base).abs().max()) / bmax
        if t % tight_every == 0 or t == nsolves:
            # and against FP64 PCG continued to a 1e-11 true relative residual
            xt = base.clone()
            torch.cuda.synchronize()
            rt = s.solve(dv(rhs), dv(xt), dmask, tol=1e-11, precision=bbpp.FP64, guess=bbpp.GUESS_GIVEN)
            tmax = float(xt.abs().max())
            for name in methods:
                rec[name][-1]["max_err_vs_tight"] = float((xs[name] - xt).abs().max()) / tmax
            rec["fp64_warm"][-1]["tight_true_rel"] = rt.true_rel
            del xt
    clk = clocks.stop()

    def summary(name):
        r = rec[name]
        ms = vmax(float(np.mean([v["ms"] for v in r])))
        tight = [v["max_err_vs_tight"] for v in r if "max_err_vs_tight" in v]
        return {"solves_per_s": aggregate(world, ms), "ms_per_solve": ms,
                "guess_ms": float(np.mean([v["guess_ms"] for v in r])),
                "iters_mean": float(np.mean([v["iters"] for v in r])), "iters_first": r[0]["iters"],
                "iters_last": r[-1]["iters"], "true_rel_max": max(v["true_rel"] for v in r),
                "max_err_vs_fp64_max": max(v["max_err_vs_fp64"] for v in r),
                "max_err_vs_tight_max": max(tight) if tight else None,
                "per_solve": [{k: (round(v, 4) if k in ("ms", "guess_ms") else v) for k, v in x.items()} for x in r]}

    res = {k: summary(k) for k in methods}
    H, B = res["learned_ir"], res["fp64_warm"]
    line = {"metric": C5_METRIC, "value": H["solves_per_s"], "unit": UNIT, "n_gpus": world, "steps": nsolves,
            "warmup": 0, "ms_per_step": H["ms_per_solve"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-inner/f64-refined (+bf16 guess)", "data": "synthetic",
            "config": {"workload": C5_WORKLOAD, "solves": nsolves,
                       "method": "learned guess from the previous pressure (C4 net, on the grid restricted by 2) + "
                                 "FP32 Jacobi PCG with FP64 reliable updates",
                       "baseline": "plain FP64 Jacobi PCG warm-started from its previous solution",
                       "l2": "not flushed: working set > 4 GB, 30x L2",
                       "rhs": "OU sequence generated on the GPU (torch generator seeded 5*7919, cuFFT), not timed"},
            "speedup_vs_fp64_warm": B["ms_per_solve"] / H["ms_per_solve"],
            "speedup_vs_ir_warm": res["ir_warm"]["ms_per_solve"] / H["ms_per_solve"],
            "methods": res, "first_solve_fp64_iters": rep0.iters, "learned_training": net_info,
            "setup_s": round(setup_s, 1), "clocks": clk,
            "gpu_launches": int(sum(v["launches"] for v in rec["learned_ir"]))}
    if rank == 0:
        print(json.dumps(line))


# forward layers of the learned guess's network: (cin, cout, n, ldi, ldo, co_off),
# n^3 volume, input channel stride ldi, output written at channel co_off of ldo
CONV_LAYERS = [(16, 16, 128, 16, 48, 32), (48, 16, 128, 48, 16, 0), (16, 16, 256, 16, 48, 32),
               (48, 16, 256, 48, 16, 0), (16, 32, 128, 16, 96, 64), (96, 32, 128, 96, 32, 0)]
CONV_KERNELS = {0: "mma_sync", 1: "tcgen05_tm", 2: "tcgen05_tx"}


def conv_layers(args):
    """Per-layer timing of the forward 3x3x3 convolution on each kernel
    (CUDA events on the launching stream, best of --steps after --warmup),
    one JSON line per layer: not the headline, the evidence for the choice of
    convolution kernel."""
    import numpy as np
    import torch
    import bbpp
    from bbpp import learned
    L = learned._sig()
    layers = CONV_LAYERS
    if args.conv_layers:
        want = [tuple(int(v) for v in spec.split(",")) for spec in args.conv_layers]
        layers = [c for c in CONV_LAYERS if c[:3] in want]
    modes = [int(m) for m in args.conv_modes.split(",")]
    for cin, cout, n, ldi, ldo, co in layers:
        rng = np.random.default_rng(cin + cout + n)
        x32 = rng.normal(size=(1, n, n, n, ldi)).astype(np.float32)
        x = (x32.view(np.uint32) >> 16).astype(np.uint16)  # BF16 bits (truncated)
        w = ((rng.normal(size=(27, cout, cin)) * 0.1).astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)
        bias = rng.normal(size=cout).astype(np.float32)
        dx, dw, db = bbpp.DeviceArray.from_host(x), bbpp.DeviceArray.from_host(w), bbpp.DeviceArray.from_host(bias)
        dy = bbpp.DeviceArray((1, n, n, n, ldo), np.uint16)
        flop = 2.0 * n ** 3 * 27 * cin * cout
        rec = {"conv_layer": "%d->%d" % (cin, cout), "n": n, "periodic": "x,y", "ms": {}, "tflops": {},
               "tcgen05_launches": {}}

        def call():
            rc = L.bbpp_conv3(cin, cout, dx.ptr, ldi, 0, dw.ptr, db.ptr, dy.ptr, ldo, co, n, n, n, 1, 1, 1, 0, 1)
            if rc != 0:
                raise RuntimeError("bbpp_conv3 returned %d" % rc)

        for mode in modes:
            assert L.bbpp_conv3_tc_config(mode, 0) == 0
            tc0 = L.bbpp_conv3_tc_launches()
            for _ in range(args.warmup):
                call()
            best = None
            for _ in range(args.steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                e0.record()  # the default stream, which bbpp_conv3 launches on
                call()
                e1.record()
                torch.cuda.synchronize()
                t = e0.elapsed_time(e1)
                best = t if best is None else min(best, t)
            name = CONV_KERNELS[mode]
            rec["ms"][name] = best
            rec["tflops"][name] = flop / (best * 1e-3) / 1e12
            rec["tcgen05_launches"][name] = L.bbpp_conv3_tc_launches() - tc0
        L.bbpp_conv3_tc_config(-1, 0)
        print(json.dumps(rec), flush=True)


def main():
    faulthandler.enable()  # a crash in native code prints the Python stack
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-learned", action="store_true", help="skip training / timing the learned guess")
    ap.add_argument("--net", default=None, help="load (or save after training) the learned-guess network here")
    ap.add_argument("--train-samples", type=int, default=2000)
    ap.add_argument("--train-steps", type=int, default=1500)
    ap.add_argument("--only", default=None, choices=["fp64", "ir", "ir_restart", "ir_every50", "ir_warm", "learned_ir",
                                                        "learned_ir_fine"],
                    help="run only warm-up + steps solves of one method (profiler runs)")
    ap.add_argument("--workload", default="C3", choices=["C3", "C5"],
                    help="C3: the headline 256^3 solve (default); C5: the 512^3 OU sequence")
    ap.add_argument("--c5-solves", type=int, default=50, help="solves of the C5 sequence")
    ap.add_argument("--conv-layers", nargs="*", default=None, metavar="CIN,COUT,N",
                    help="time the forward convolution layers (all, or the ones named) on each kernel instead")
    ap.add_argument("--conv-modes", default="0,1,2", help="convolution kernels to time (0 mma.sync, 1 tm, 2 tx)")
    args = ap.parse_args()
    args.steps = max(1, args.steps)
    if args.conv_layers is not None:
        conv_layers(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "C5":
        run_c5(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
