"""Benchmark: simulated ns per wall-second of nmag's LLG path on the film.

Default line: the chosen form -- an ensemble of 8 films on the one mesh
(options n_members = 8), BEM matrix as FP32 + BF16 residual with compensated
FP32 products (accurate to ~2^-44), Poisson CG iterating in FP32 with FP64
residual refinement to the same tolerance -- with
`value` summed over the members, and beside it (`plain_fp64`) the plain FP64
single film measured in the same run, their ratio and the chosen form's
H_eff error against FP64 at the same magnetisation.  `--form fp64
--members 1` measures the plain form alone.

Workload (the plain-method film configuration): 500 x 125 x 3 nm permalloy
film, 2.5 x 2.5 x 1.5 nm cells, Kuhn 6-tet split (30,753 nodes, 120,000
tets, 21,002 boundary nodes, dense 21,002^2 BEM = 3.53 GB FP64), alpha = 0.02,
gamma = 2.211e5 m/(A s), uniform H_ext = (-24.6, 4.3, 0) mT / mu0, BDF
rtol = atol = 1e-6.  Inputs are synthetic (numpy default_rng(1) initial m).
A step advances the simulation by 1 ps (the recording interval) and reads
<m>; the BEM (3.5 GB) is larger than L2, so every step streams it from HBM.

Our arm: the library through nmag.Simulation (e2e: advance_time + m copied to
the host each call, like the reference's master buffer) and the same steps
on the device-resident engine (value: CUDA-event time on the library's
stream).  --impl reference: the CPU restatement of the reference's path
(oracle/, all host cores) on the same workload and metric.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                       [--form fp64|fp32] [--members B] [--cg fp64|fp32] [--no-compare]
                       [--workload film|cube|film_small]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np


def _pin_rank_device():
    """Under torchrun each rank sees only its own GPU (set before any CUDA
    initialisation): the library links the CUDA runtime statically, so its
    current device does not follow torch.cuda.set_device."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = os.environ.get("LOCAL_RANK")
    if world > 1 and local is not None and "NMAG_BENCH_PINNED" not in os.environ:
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        devices = [d for d in vis.split(",") if d] if vis else [str(i) for i in range(64)]
        os.environ["CUDA_VISIBLE_DEVICES"] = devices[int(local) % len(devices)]
        os.environ["NMAG_BENCH_PINNED"] = "1"
        os.environ["LOCAL_RANK_DEVICE"] = "0"


_pin_rank_device()

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "nmag-src_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

MU0 = 4e-7 * np.pi
H_EXT_MT = (-24.6, 4.3, 0.0)

# DRAM bytes per launch of the BEM product divided by its algorithmic bytes,
# from ncu captures on the 8,562-boundary-node profiling film (matrices larger
# than L2; profiles/k_gemv_f64_film_small.txt: 590.63 MB read+written for
# 586.6 MB).  The traffic grows with the matrix entries, so it scales to the
# full film.
NCU_TRAFFIC_RATIO = {("fp64", False): (587.56 + 3.07) / 586.60,
                     # k_gemv_df, profiling film, one film: 441.09 + 2.80 MB of 439.98 MB algorithmic
                     # (profiles/k_gemv_df_film_small.txt)
                     ("fp32x2", False): (441.09 + 2.80) / 439.98,
                     # k_gemm_df<8>, profiling film, 8 members: 440.75 + 6.60 MB of 440.95 MB algorithmic
                     # (profiles/k_gemm_df_film_small_ensemble.txt)
                     ("fp32x2", True): (440.75 + 6.60) / 440.95}
# the same figures keyed by kernel (the anchored product reports whichever of
# its two kernels dominates)
NCU_TRAFFIC_RATIO[("k_gemv_df", False)] = NCU_TRAFFIC_RATIO[("fp32x2", False)]
NCU_TRAFFIC_RATIO[("k_gemm_df", True)] = NCU_TRAFFIC_RATIO[("fp32x2", True)]
# k_gemm_f32r<8> (anchored difference product), profiling film, 8 members: 293.80 + 3.54 MB of
# 294.30 MB algorithmic (profiles/k_gemm_f32r_film_small_ensemble.txt)
NCU_TRAFFIC_RATIO[("k_gemm_f32r", True)] = (293.80 + 3.54) / 294.30


def workload(name):
    from nmag import mesh
    if name == "film":
        return mesh.film_mesh(), (1.0, 0.25, 0.1), 1
    if name == "cube":
        return mesh.cube_mesh(), (1.0, 1.0, 1.0), 0
    if name == "film_small":
        return mesh.box_mesh(100, 40, 2, 2.5, 2.5, 1.5), (1.0, 0.25, 0.1), 1
    raise ValueError(name)


def initial_m(n, base, seed):
    rng = np.random.default_rng(seed)
    m = np.asarray(base)[None, :] + 0.01 * rng.standard_normal((n, 3))
    return m / np.linalg.norm(m, axis=1)[:, None]


def material(alpha):
    import nmag
    from nmag import SI
    return nmag.MagMaterial("Py", Ms=SI(8.6e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"), llg_damping=alpha,
                            llg_gamma_G=SI(2.211e5, "m/A s"))


def h_ext_su():
    # mu0 H in mT -> H in A/m -> simulation units (1e6 A/m)
    return np.array([v * 1e-3 / MU0 for v in H_EXT_MT]) / 1e6


def ksp_tolerances(args):
    """The Poisson solves' tolerances: the reference's defaults (rtol 1e-5,
    main.py ksp_tolerances) unless --poisson-rtol is given."""
    if args.poisson_rtol is None:
        return None
    return {"NBC.rtol": args.poisson_rtol, "DBC.rtol": args.poisson_rtol}


def oracle_tolerances(args):
    """The same for the CPU legs (the oracle's (rtol, atol, maxits))."""
    tol = 1e-5 if args.poisson_rtol is None else args.poisson_rtol
    return (tol, 1e-50, 10000), (tol, 1e-50, 10000)


def peaks_tensor():
    """Dense bf16 tensor peak (TFLOP/s): the measured burst figure, else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler(object):
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("NMAG_BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return rank, world


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_reference_run(args, msh, base, seed, steps, warmup, max_wall=25.0, sample_ps=None):
    """Time the oracle (CPU restatement, all host threads) on a bounded
    sample of the workload: the seeded state relaxed at alpha = 1 without
    field for args.relax_ps (the full relaxation to 1 deg/ns would take the
    CPU longer than the whole run may), then alpha = 0.02 under H_ext,
    `warmup` untimed records and up to `steps` timed records of sample_ps
    (default: record_ps), stopping early after max_wall seconds."""
    import oracle
    t0 = time.perf_counter()
    om = oracle.OracleMesh(msh.points, msh.simplices, nthreads=0)
    m = initial_m(msh.n_nodes, base, seed)
    if args.relax_ps > 0:
        nbc, dbc = oracle_tolerances(args)
        r = oracle.OracleSim(om, material(1.0).coefficients("nmag"), nbc=nbc, dbc=dbc)
        r.ts_init(m, rtol=1e-6, atol=1e-6)
        _, m = r.ts_advance(args.relax_ps)
        del r
    nbc, dbc = oracle_tolerances(args)
    s = oracle.OracleSim(om, material(0.02).coefficients("nmag"), nbc=nbc, dbc=dbc)
    s.set_h_ext(h_ext_su())
    s.ts_init(m, rtol=1e-6, atol=1e-6)
    setup = time.perf_counter() - t0
    t = 0.0
    dt = sample_ps or args.record_ps
    for _ in range(warmup):
        t += dt
        s.ts_advance(t)
    nfe0 = s.ts_stats()["nfe"]
    done, wall = 0.0, 0.0
    n = 0
    while n < steps:
        t += dt
        a = time.perf_counter()
        s.ts_advance(t)
        wall += time.perf_counter() - a
        done += dt
        n += 1
        if wall > max_wall:
            break
    st = s.ts_stats()
    return {"sim_ps": done, "wall_s": wall, "steps": n, "nfe": st["nfe"] - nfe0, "setup_s": setup,
            "cores": os.cpu_count(), "dt": dt}


def run_reference(args):
    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    msh, base, seed = workload(args.workload)
    r = cpu_reference_run(args, msh, base, seed, args.steps, args.warmup, max_wall=150.0)
    value = (r["sim_ps"] * 1e-3) / r["wall_s"]
    line = {
        "impl": "reference", "metric": "simulated ns/wall-s", "value": value, "unit": "ns/s",
        "n_gpus": args.gpus, "steps": r["steps"], "warmup": args.warmup,
        "ms_per_step": 1e3 * r["wall_s"] / max(r["steps"], 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(args, msh),
        "rhs_evals_per_s": r["nfe"] / r["wall_s"],
        "cpu_baseline": {"value": value, "unit": "ns/s", "cores": r["cores"], "kind": "port",
                         "sample": "%d x %.2f ps records of the workload's dynamics on the CPU restatement "
                                   "(oracle/, OpenMP), after a %g ps relax at alpha=1 (the relax to 1 deg/ns "
                                   "is beyond a bounded CPU run)" % (r["steps"], r["dt"], args.relax_ps)},
        "e2e": {"value": value, "unit": "ns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own build (OCaml/Python 2/PETSc/SUNDIALS) cannot run here; this arm times "
                "the CPU restatement of its algorithms (FP64).  An ensemble's members would run one after "
                "another on the CPU, so its aggregate rate equals this single-film rate",
    }
    print(json.dumps(line))


WORKLOAD_NAMES = {
    "film": "film 500x125x3 nm, 30753 nodes, 21002 boundary nodes, alpha 0.02, H_ext (-24.6,4.3,0) mT",
    "cube": "cube 30 nm, 1331 nodes, 602 boundary nodes",
    "film_small": "film 250x100x3 nm (profiling size), 12423 nodes, 8562 boundary nodes, alpha 0.02",
}


def config_dict(args, msh):
    return {"workload": WORKLOAD_NAMES[args.workload],
            "relax": ("alpha=1, H_ext=0, nmag relax() until max |dm/dt| < 1 deg/ns twice in a row (checked every "
                      "5 BDF steps; capped at %g ps), untimed; the timed dynamics start from the relaxed state"
                      % args.relax_cap_ps),
            "nodes": int(msh.n_nodes), "tets": int(msh.n_tets),
            "step": "%g ps advance in %g ps records, each followed by an <m> read" % (args.step_ps, args.record_ps),
            "interval_ps": args.steps * args.step_ps,
            "form": args.form, "cg": args.cg, "cg_local_sweeps": args.cg_sweeps, "members": args.members,
            "jv": args.jv, "cg_coarse": not args.cg_no_coarse,
            "bem_anchor": args.anchor if args.form == "fp32x2" else 0.0,
            "rtol": 1e-6, "atol": 1e-6, "max_order": 2, "krylov_max": 300,
            "poisson_rtol": 1e-5 if args.poisson_rtol is None else args.poisson_rtol,
            "l2": "BEM matrix (nb^2 x %d B) larger than L2; no explicit flush" % {"fp64": 8, "fp32": 4,
                                                                                  "fp32x2": 6, "bf16x3": 6}[args.form]}


# records (1-based, in record_ps units) where the e2e leg keeps WINDOW_LEN
# consecutive states for the anchored product's error walk
WINDOW_RECORDS = (100, 500, 900)
WINDOW_LEN = 6


def relax_states(args, form, cg, B, msh, base, seed, anchor):
    """The workload's relaxation, untimed: each member's seeded initial state
    relaxed at alpha = 1 without field by nmag's own relax() -- integrate,
    check max |dm/dt| every 5 steps, stop once it is below 1 deg/ns twice in
    a row (convergence.py:54-100, hysteresis.py:207-242) -- capped at
    args.relax_cap_ps of simulated time.  Returns the relaxed states and a
    record of the relaxation."""
    import nmag
    from nmag import SI, every
    sim = nmag.Simulation("relax", bem_precision=form, cg_precision=cg, n_members=B, bem_anchor=anchor,
                          anchor_product=args.anchor_product, cg_local_sweeps=args.cg_sweeps,
                          ksp_tolerances=ksp_tolerances(args))
    sim.load_mesh(msh, [("film", material(1.0))], unit_length=SI(1e-9, "m"))
    if B > 1:   # member b starts from the workload's initial state with seed + b
        sim.set_m(np.stack([initial_m(msh.n_nodes, base, seed + b) for b in range(B)]))
    else:
        sim.set_m(initial_m(msh.n_nodes, base, seed))
    cap = args.relax_cap_ps

    def stop_at_cap(s):
        if s.clock.stage_time_su >= cap:
            s.hysteresis_exit(s)

    w = time.perf_counter()
    sim.relax(save=(), do=((stop_at_cap, every("step", 5)),))
    wall = time.perf_counter() - w
    rec = {"sim_ps": float(sim.clock.stage_time_su), "wall_s": wall, "bdf_steps": int(sim.clock.stage_step),
           "converged": bool(sim.clock.convergence), "final_max_dm_dt_deg_per_ns": float(sim.max_dm_dt) / 1.7453292519943296e-05,
           "form": form if B > 1 or form != "fp64" else "fp64", "members": B}
    m = sim.engine.get_m()
    sim.engine.close()
    return m, rec


def measure(args, form, cg, B, msh, start, world, local, sample_clocks=True, anchor=0.0, warmup=None,
            e2e=True, jacobian="approximate", jv=None):
    """One form on the workload from the relaxed states `start`: alpha =
    0.02 and the applied field; W untimed warm-up steps, then the state is
    put back and K timed steps run on the device-resident engine (value:
    CUDA-event time of the advances on the library's stream), then the state
    is put back again and the same K steps run through nmag.Simulation (e2e:
    advance_time, which copies m to the host, and <m> read on the host).  A
    step advances step_ps in records of record_ps, each followed by an <m>
    read, so K steps from t = 0 cover exactly the configured interval."""
    import torch
    import nmag
    from nmag import SI
    sim = nmag.Simulation("bench", bem_precision=form, cg_precision=cg, n_members=B, bem_anchor=anchor,
                          anchor_product=args.anchor_product, cg_local_sweeps=args.cg_sweeps,
                          jacobian=jacobian, jacobian_demag_rtol=args.jac_rtol,
                          jv_precision=jv if jv is not None else args.jv, cg_coarse=not args.cg_no_coarse,
                          ksp_tolerances=ksp_tolerances(args))
    sim.load_mesh(msh, [("film", material(0.02))], unit_length=SI(1e-9, "m"))
    eng = sim.engine
    sim.set_H_ext(h_ext_su() * 1e6, SI(1.0, "A/m"))
    rec = args.record_ps
    per_step = int(round(args.step_ps / rec))
    warmup = args.warmup if warmup is None else warmup

    def restart():
        sim.set_m(start)
        sim.reinitialise(initial_time=0)

    restart()
    t = 0.0
    for _ in range(warmup * per_step):
        t += rec
        eng.ts_advance(t)
        eng.averages()
    restart()
    t = 0.0
    # ---- timed region: device-resident value leg ----
    sampler = ClockSampler(local) if sample_clocks else None
    if sampler:
        sampler.start()
    eng.profile(True)
    launches0 = eng.launch_count()
    cg0 = eng.cg_iterations()
    anc0 = eng.bem_anchor_stats()
    _, st0 = eng.ts_advance(t)   # no-op advance to read the counters
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    dev_ms = 0.0
    trace = []
    torch.cuda.nvtx.range_push("timed")   # lets a profiler capture the timed region alone
    w0 = time.perf_counter()
    for _ in range(args.steps):
        for _ in range(per_step):
            t += rec
            _, st = eng.ts_advance(t)
            dev_ms += float(eng.timings()[0])
            trace.append(eng.averages())
    torch.cuda.synchronize()
    wall_value = time.perf_counter() - w0
    torch.cuda.nvtx.range_pop()
    barrier(world)
    launches = eng.launch_count() - launches0
    cg1 = eng.cg_iterations()
    anc1 = eng.bem_anchor_stats()
    eng.profile(False)
    prof = eng.profile_read()
    clocks = sampler.stop() if sampler else None
    m_final = eng.get_m()
    # ---- e2e leg through the public API, over the same interval from the same state ----
    wall_e2e = None
    windows = []
    if e2e:
        restart()
        torch.cuda.synchronize()
        barrier(world)
        w1 = time.perf_counter()
        t = 0.0
        keep = {k for first in WINDOW_RECORDS for k in range(first, first + WINDOW_LEN)}
        snaps = {}
        nrec = 0
        for _ in range(args.steps):
            for _ in range(per_step):
                t += rec
                sim.advance_time(SI(t * 1e-12, "s"))
                sim.get_subfield_average_siv("m")
                nrec += 1
                if anchor > 0 and nrec in keep:   # m is on the host already (advance_time copied it)
                    snaps[nrec] = np.array(sim._m, copy=True)
        torch.cuda.synchronize()
        wall_e2e = max_over_ranks(time.perf_counter() - w1, world)
        windows = [[snaps[k] for k in range(first, first + WINDOW_LEN) if k in snaps] for first in WINDOW_RECORDS]
        windows = [w for w in windows if len(w) >= 2]
    dev_s = max_over_ranks(dev_ms * 1e-3, world)
    sim_ns_total = world * B * args.steps * args.step_ps * 1e-3   # summed over ensemble members
    nb = eng.nb
    elem = {"fp64": 8, "fp32": 4, "fp32x2": 6, "bf16x3": 6}[form]
    nm = min(B, 8)   # members per BEM launch
    gl, gms = prof["bem_gemv"]
    bytes_per_launch = nb * nb * elem + 2 * nm * nb * 8
    roof = None
    if gl > 0:
        hbm, peak_kind = peaks()
        avg_ms = gms / gl
        achieved = bytes_per_launch / (avg_ms * 1e-3) / 1e9
        if B == 1:
            kname = {"fp64": "k_gemv_f64", "fp32": "k_gemv_f32", "fp32x2": "k_gemv_df"}[form]
        else:
            kname = {"fp64": "k_gemm_f64", "fp32": "k_gemm_f32r", "fp32x2": "k_gemm_df"}[form]
        roof = {"bound": "hbm" if not (B > 1 and form == "fp64") else "fp64 pipe (bytes shown)",
                "kernel": kname, "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "peak_kind": peak_kind,
                "traffic": (NCU_TRAFFIC_RATIO[(form, B > 1)] * bytes_per_launch / 1e9
                            if (form, B > 1) in NCU_TRAFFIC_RATIO else None),
                "traffic_unit": "GB per launch (ncu dram__bytes_read+write, scaled from the profiling capture)",
                "launches": gl, "avg_launch_ms": avg_ms,
                "algorithmic_bytes_per_launch": bytes_per_launch,
                "share_of_step": gms / max(dev_ms, 1e-9)}
        if form == "fp32x2" and B > 1:
            roof["note"] = ("compute-bound on the FP32 pipe (~11 FP32 ops per member-entry; ncu: FMA pipe 71.5% "
                            "active, profiles/k_gemm_df_film_small_ensemble.txt); the HBM fraction is shown")
    anchored = None
    if anchor > 0:
        # two gated kernels per chunk product: the compensated one runs on a
        # refresh, the FP32 difference product otherwise (the other exits at
        # once; its launch time stays in the totals)
        n_prod, n_ref = anc1[0] - anc0[0], anc1[1] - anc0[1]
        dl, dms = prof["bem_anchor_delta"]
        h16 = B > 1 and args.anchor_product == "fp16"
        # difference product: the FP32 matrix, or the FP16 fragment copy (16 x 16
        # tiles covering nb rounded up to 16); x - x0 in and y out per member
        kt = (nb + 15) // 16
        bytes_d = (kt * kt * 512 if h16 else nb * nb * 4) + 2 * nm * nb * 8
        hbm, peak_kind = peaks()
        legs = {}
        for name, kname, execd, tot_ms, nbytes in (
                ("refresh", "k_gemm_df" if B > 1 else "k_gemv_df", n_ref, gms, bytes_per_launch),
                ("difference", ("k_gemm_h16mma" if h16 else "k_gemm_f32r") if B > 1 else "k_gemv_f32",
                 n_prod - n_ref, dms, bytes_d)):
            ach = execd * nbytes / (tot_ms * 1e-3) / 1e9 if execd > 0 and tot_ms > 0 else None
            legs[name] = {"kernel": kname, "executed": int(execd), "total_ms": tot_ms,
                          "algorithmic_bytes_per_launch": nbytes,
                          "avg_launch_ms": tot_ms / execd if execd > 0 else None,
                          "achieved": ach, "frac": ach / hbm if ach else None}
        anchored = {"tol": anchor, "products": int(n_prod), "refreshes": int(n_ref), "legs": legs,
                    "difference_product": "fp16 fragments (mma.m16n8k16)" if h16 else "fp32"}
        dom = max(legs.values(), key=lambda v: v["total_ms"])
        if dom["achieved"]:
            roof = {"bound": "hbm" if dom["kernel"] in ("k_gemm_f32r", "k_gemv_f32", "k_gemm_h16mma") else "hbm (FP32 pipe)",
                    "kernel": dom["kernel"], "achieved": dom["achieved"], "peak": hbm, "unit": "GB/s",
                    "frac": dom["frac"], "peak_kind": peak_kind,
                    "traffic": (NCU_TRAFFIC_RATIO[(dom["kernel"], B > 1)] * dom["algorithmic_bytes_per_launch"] / 1e9
                                if (dom["kernel"], B > 1) in NCU_TRAFFIC_RATIO else None),
                    "traffic_unit": "GB per launch (ncu dram__bytes_read+write, scaled from the profiling capture)",
                    "launches": dom["executed"], "avg_launch_ms": dom["avg_launch_ms"],
                    "algorithmic_bytes_per_launch": dom["algorithmic_bytes_per_launch"],
                    "share_of_step": dom["total_ms"] / max(dev_ms, 1e-9),
                    "note": "anchored product: the larger of its two kernels (both in 'anchored'); the BEM "
                            "product is the largest HBM-streaming kernel of the step -- see dominant_kernel "
                            "for the largest by time"}
    # the largest kernel by device time over the timed steps, with its share
    kms = {k: v for k, v in prof.items() if v[0] > 0}
    dominant = None
    if kms:
        top = max(kms, key=lambda k: kms[k][1])
        dominant = {"slot": top, "total_ms": kms[top][1], "launches": kms[top][0],
                    "share_of_step": kms[top][1] / max(dev_ms, 1e-9)}
        if top == "cg_neumann":
            its = cg1[0] - cg0[0]
            dominant.update({
                "kernel": "k_cgm_mp" if cg == "fp32" else ("k_cgm" if B > 1 else "k_cg3"),
                "inner_iterations": int(its), "us_per_iteration": 1e3 * kms[top][1] / max(its, 1),
                "bound": "latency: two grid barriers and their block reductions per inner iteration; the "
                         "CSR rows sit in shared memory and the exchanged vectors (~2 MB per iteration for "
                         "8 members) in L2, so DRAM is idle (ncu: profiles/k_cgm_mp_film_small_ensemble.txt)"})
    return {
        "sim": sim, "eng": eng, "value": sim_ns_total / dev_s, "dominant_kernel": dominant,
        "e2e": sim_ns_total / wall_e2e if wall_e2e else None,
        "ms_per_step": dev_s * 1e3 / args.steps, "rhs_evals": st["nfe"] - st0["nfe"],
        "bdf_steps": st["nst"] - st0["nst"], "rhs_evals_per_s": (st["nfe"] - st0["nfe"]) / dev_s * world,
        "newton": {k: st[k] - st0[k] for k in ("nni", "nli", "ncfn", "netf", "njv", "npe")},
        "wall_value_s": wall_value, "roofline": roof, "launches": launches, "clocks": clocks,
        "kernels_ms": {k: {"launches": v[0], "total_ms": v[1]} for k, v in prof.items()},
        "cg_iterations": {"neumann": cg1[0] - cg0[0], "dirichlet": cg1[1] - cg0[1]},
        # per step: B members' m copied to the host (advance_time) + <m> (24 B) per record
        "d2h": per_step * (B * msh.n_nodes * 3 * 8 + 24),
        "anchored": anchored, "m_start": start, "m_final": m_final, "trace": np.asarray(trace),
        "windows": windows,
    }


def heff_error(args, chosen, msh):
    """Relative H_eff error of the chosen form against FP64 at the same
    magnetisation (member 0 after the timed steps): max |H - H_fp64| /
    max |H_fp64|.  Both sides are fresh handles whose Poisson solves are
    converged to rtol 1e-12, so the figure is the form's own error (FP32
    matrix entries), not the difference of two CG solves stopped at the
    reference's default tolerance."""
    import nmag
    from nmag import SI
    m = chosen["eng"].get_m()
    m0 = m[0] if m.ndim == 3 else m
    tight = {"NBC.rtol": 1e-12, "DBC.rtol": 1e-12, "NBC.maxits": 20000, "DBC.maxits": 20000}
    out = {}
    for form in (args.form, "fp64"):
        sim = nmag.Simulation("err", bem_precision=form, ksp_tolerances=tight)
        sim.load_mesh(msh, [("film", material(0.02))], unit_length=SI(1e-9, "m"))
        sim.engine.set_m(m0)
        sim.engine.set_h_ext(np.broadcast_to(h_ext_su(), (sim.engine.N, 3)))
        out[form] = sim.engine.eval_fields()["H_total"]
        sim.engine.close()
    ref = out["fp64"]
    return float(np.abs(out[args.form] - ref).max() / np.abs(ref).max())


def anchor_path_error(args, chosen, msh, blends=4):
    """H_eff error of the anchored product along the run's own trajectory.
    The e2e leg keeps the members' states of a few windows of consecutive
    records (chosen["windows"]); each window is walked in order, with
    `blends` normalised linear blends per record interval, through the
    anchored form (its anchor carried along, so most products are FP32
    differences from an earlier state, a refresh when the drift passes tol)
    and through the FP64 form; both converge their Poisson solves to 1e-12.
    Returns the max over the walk and the members of max |H - H_fp64| /
    max |H_fp64|, the anchor's product / refresh counts over the walk and
    the number of evaluations."""
    import nmag
    from nmag import SI
    B = args.members
    tight = {"NBC.rtol": 1e-12, "DBC.rtol": 1e-12, "NBC.maxits": 20000, "DBC.maxits": 20000}
    sims = {}
    for key, form, anc in (("anchored", args.form, args.anchor), ("fp64", "fp64", 0.0)):
        sim = nmag.Simulation("err", bem_precision=form, ksp_tolerances=tight, n_members=B, bem_anchor=anc,
                              anchor_product=args.anchor_product, cg_local_sweeps=args.cg_sweeps)
        sim.load_mesh(msh, [("film", material(0.02))], unit_length=SI(1e-9, "m"))
        shape = (B, sim.engine.N, 3) if B > 1 else (sim.engine.N, 3)
        sim.engine.set_h_ext(np.broadcast_to(h_ext_su(), shape))
        sims[key] = (sim, shape)
    worst, evals = 0.0, 0
    for window in chosen["windows"]:
        states = [np.asarray(w).reshape(B, -1, 3) for w in window]
        path = []
        for a, b in zip(states[:-1], states[1:]):
            for j in range(blends):
                path.append((1.0 - j / blends) * a + (j / blends) * b)
        path.append(states[-1])
        for m in path:
            m = m / np.linalg.norm(m, axis=-1, keepdims=True)
            H = {}
            for key, (sim, shape) in sims.items():
                sim.engine.set_m(m.reshape(shape))
                H[key] = np.asarray(sim.engine.eval_fields()["H_total"]).reshape(B, -1, 3)
            for b in range(B):
                ref = H["fp64"][b]
                worst = max(worst, float(np.abs(H["anchored"][b] - ref).max() / np.abs(ref).max()))
            evals += 1
    prod, ref_n = sims["anchored"][0].engine.bem_anchor_stats()
    for sim, _ in sims.values():
        sim.engine.close()
    return worst, prod, ref_n, evals


def run_precision_report(args):
    """Precision form against FP64 on the film for N seeded random fields
    (m = normalise(N(0,1)) per node, numpy default_rng(seed), seeds 100..):
    H_eff (max-norm relative) and total / demag energy relative errors.  Both
    sides are ensembles (--precision-members fields each; every field of an
    ensemble goes through one BEM product) with Poisson solves converged to
    1e-12; the FP64 side is the plain form's arithmetic.  For the tensor-core
    form (bf16x3) the BEM products are timed with CUDA events and reported
    against the measured bf16 tensor peak."""
    import torch
    import nmag
    from nmag import SI
    torch.cuda.set_device(0)
    msh, _, _ = workload(args.workload)
    tight = {"NBC.rtol": 1e-12, "DBC.rtol": 1e-12, "NBC.maxits": 20000, "DBC.maxits": 20000}
    B = args.precision_members or (128 if args.form == "bf16x3" else 8)
    sims = {}
    for form in (args.form, "fp64"):
        sim = nmag.Simulation("err", bem_precision=form, ksp_tolerances=tight, n_members=B)
        sim.load_mesh(msh, [("film", material(0.02))], unit_length=SI(1e-9, "m"))
        sim.engine.set_h_ext(np.broadcast_to(h_ext_su(), (B, sim.engine.N, 3)))
        sims[form] = sim.engine
    sims[args.form].profile(True)
    N = msh.n_nodes
    herr, eerr, derr = [], [], []
    t0 = time.perf_counter()
    for s0 in range(100, 100 + args.fields, B):
        seeds = list(range(s0, min(s0 + B, 100 + args.fields)))
        ms = []
        for sd in seeds:
            g = np.random.default_rng(sd).standard_normal((N, 3))
            ms.append(g / np.linalg.norm(g, axis=1)[:, None])
        while len(ms) < B:
            ms.append(ms[-1])
        res = {}
        for form, eng in sims.items():
            eng.set_m(np.stack(ms))
            f = eng.eval_fields()["H_total"]
            en = [eng.member_averages(b, energies=True)[1] for b in range(len(seeds))]
            res[form] = (f, en)
        for b in range(len(seeds)):
            h32, h64 = res[args.form][0][b], res["fp64"][0][b]
            herr.append(float(np.abs(h32 - h64).max() / np.abs(h64).max()))
            e32, e64 = res[args.form][1][b], res["fp64"][1][b]
            eerr.append(float(abs(e32[4] - e64[4]) / abs(e64[4])))
            derr.append(float(abs(e32[1] - e64[1]) / abs(e64[1])))
    wall = time.perf_counter() - t0
    eng = sims[args.form]
    eng.profile(False)
    launches, ms_tot = eng.profile_read()["bem_gemv"]
    line = {"metric": "precision form error vs FP64", "report": "precision", "fields": len(herr),
            "seeds": [100, 100 + len(herr) - 1], "workload": WORKLOAD_NAMES[args.workload],
            "form": args.form, "members_per_product": B, "bound": 1e-5,
            "heff_rel_err": {"max": max(herr), "median": float(np.median(herr)), "p99": float(np.percentile(herr, 99))},
            "energy_total_rel_err": {"max": max(eerr), "median": float(np.median(eerr))},
            "energy_demag_rel_err": {"max": max(derr), "median": float(np.median(derr))},
            "within_bound": bool(max(herr) <= 1e-5), "wall_s": wall}
    if launches:
        nb = eng.nb
        avg_ms = ms_tot / launches
        line["bem_product"] = {"kernel": {"bf16x3": "k_bem_tc", "fp32x2": "k_gemm_df", "fp32": "k_gemm_f32r",
                                          "fp64": "k_gemm_f64"}[args.form],
                               "launches": launches, "avg_launch_ms": avg_ms,
                               "right_hand_sides_per_launch": B,
                               "fields_per_s": B / (avg_ms * 1e-3)}
        if args.form == "bf16x3":
            flop = 6 * 2.0 * nb * nb * B   # six BF16 products per term on the tensor pipe
            peak = peaks_tensor()
            line["bem_product"]["roofline"] = {
                "bound": "tensor", "achieved": flop / (avg_ms * 1e-3) / 1e12, "peak": peak[0], "unit": "TFLOP/s",
                "frac": flop / (avg_ms * 1e-3) / 1e12 / peak[0], "peak_kind": peak[1],
                "flop_per_launch": flop, "algorithmic_flop_per_launch": 2.0 * nb * nb * B,
                "note": "tensor FLOPs = 6 split products x 2 nb^2 R; the product itself is 2 nb^2 R"}
    print(json.dumps(line))


def run_bem_report(args):
    """The BEM product alone: y_n = B x_n for --rhs right-hand sides (smooth
    boundary potentials of different wavelengths) in the chosen form, W
    warm-up products, then K timed products (CUDA events around the product
    kernel on the library's stream); error against the FP64 product of the
    same vectors; tensor-pipe (bf16x3) or HBM fraction of the measured peaks."""
    import torch
    import nmag
    from nmag import SI
    torch.cuda.set_device(0)
    msh, _, _ = workload(args.workload)
    engines = {}
    for form in dict.fromkeys((args.form, "fp64")):
        sim = nmag.Simulation("bem", bem_precision=form)
        sim.load_mesh(msh, [("film", material(0.02))], unit_length=SI(1e-9, "m"))
        engines[form] = sim.engine
    eng = engines[args.form]
    nb, R = eng.nb, args.rhs
    k = np.arange(nb)
    X = np.stack([100.0 * np.sin(k * w + ph) for ph, w in enumerate(np.geomspace(1e-4, 3e-1, R))])
    dx = torch.tensor(X, dtype=torch.float64, device="cuda")
    dy = torch.empty_like(dx)
    dr = torch.empty_like(dx)
    engines["fp64"].bem_apply_device(dx.data_ptr(), dr.data_ptr(), R)
    for _ in range(args.warmup):
        eng.bem_apply_device(dx.data_ptr(), dy.data_ptr(), R)
    torch.cuda.synchronize()
    eng.profile(True)
    w = time.perf_counter()
    for _ in range(args.steps):
        eng.bem_apply_device(dx.data_ptr(), dy.data_ptr(), R)
    wall = time.perf_counter() - w
    eng.profile(False)
    launches, ms_tot = eng.profile_read()["bem_gemv"]
    err = float((dy - dr).abs().max() / dr.abs().max())
    avg_ms = ms_tot / max(launches, 1)
    line = {"metric": "BEM product", "report": "bem", "workload": WORKLOAD_NAMES[args.workload], "nb": nb,
            "form": args.form, "right_hand_sides": R, "steps": args.steps, "warmup": args.warmup,
            "profiled_launches": launches, "avg_launch_ms": avg_ms, "wall_ms_per_product": 1e3 * wall / args.steps,
            "rel_err_vs_fp64": err}
    if args.form == "bf16x3":
        flop = 6 * 2.0 * nb * nb * R
        peak, kind = peaks_tensor()
        line["roofline"] = {"bound": "tensor", "achieved": flop / (avg_ms * 1e-3) / 1e12, "peak": peak,
                            "unit": "TFLOP/s", "frac": flop / (avg_ms * 1e-3) / 1e12 / peak, "peak_kind": kind,
                            "flop_per_launch": flop,
                            "bytes_per_launch": 3 * 2.0 * nb * nb + 3 * 2.0 * nb * R,
                            "note": "six BF16 tensor products per term (tensor FLOPs = 6 x 2 nb^2 R)"}
    else:
        elem = {"fp64": 8, "fp32": 4, "fp32x2": 6}[args.form]
        hbm, kind = peaks()
        nbytes = elem * nb * nb * R + 16 * nb * R
        line["roofline"] = {"bound": "hbm", "achieved": nbytes / (avg_ms * 1e-3) / 1e9, "peak": hbm,
                            "unit": "GB/s", "frac": nbytes / (avg_ms * 1e-3) / 1e9 / hbm, "peak_kind": kind,
                            "note": "one product per vector (the single-film kernels)"}
    print(json.dumps(line))


def run_adjoint_report(args):
    """Differentiation form on the workload: fixed-step RK4 (dt = 0.1 ps) with
    per-element Ms (Ms (1 + 0.05 N(0,1)), seed 3), per-element K1 (0) and 20
    pulse amplitudes (N(0, 5 mT), seed 4) as parameters, loss
    ||<m>(T) - (0,1,0)||^2 + 1e-3 mean_t <m>_x^2; times one forward + adjoint
    (CUDA-event free: wall time around synchronised calls) and checks the
    adjoint's directional derivatives against central differences
    (h = 1e-6 relative) along seeded directions on a shorter trajectory."""
    import torch
    import nmag
    from nmag import SI, adjoint
    torch.cuda.set_device(0)
    msh, base, seed = workload(args.workload)
    mat = material(0.02)
    sim = nmag.Simulation("adj", ksp_tolerances={"NBC.rtol": args.adj_ksp, "DBC.rtol": args.adj_ksp},
                          bem_precision=args.adj_form, cg_precision=args.adj_cg,
                          adjoint_cg_precision=args.adj_bwd_cg)
    sim.load_mesh(msh, [("film", mat)], unit_length=SI(1e-9, "m"))
    eng = sim.engine
    c = mat.coefficients("nmag")
    from nmag.si import simulation_units, mu0 as mu0_si
    mu0 = simulation_units.of(mu0_si)
    T = eng.T
    Ms_T = c["Ms"] * (1.0 + 0.05 * np.random.default_rng(3).standard_normal(T))
    K1_T = np.zeros(T)
    pulses = np.random.default_rng(4).standard_normal((20, 3)) * (5e-3 / MU0) * 1e-6
    m0 = initial_m(msh.n_nodes, base, seed).reshape(-1)
    eng.set_h_ext(np.broadcast_to(h_ext_su(), (eng.N, 3)))
    dt = 0.1
    nsteps, ckpt = args.adj_steps, 50
    spp = max(1, nsteps // 20)
    axis = (1.0, 0.0, 0.0)

    def run(Ms, K1, P, steps, grad):
        tM = torch.tensor(Ms, device="cuda", dtype=torch.float64, requires_grad=grad)
        tK = torch.tensor(K1, device="cuda", dtype=torch.float64, requires_grad=grad)
        tP = torch.tensor(P, device="cuda", dtype=torch.float64, requires_grad=grad)
        tm = torch.tensor(m0, device="cuda", dtype=torch.float64)
        _, hist = adjoint.rk4_trajectory(eng, tm, tM, tK, tP, axis, c["Ms"], mu0, dt, steps, ckpt,
                                         max(1, steps // 20))
        loss = adjoint.film_loss(hist)
        if grad:
            loss.backward()
            return loss.item(), tM.grad.cpu().numpy(), tK.grad.cpu().numpy(), tP.grad.cpu().numpy()
        return loss.item()

    torch.cuda.synchronize()
    launches0 = eng.launch_count()
    w = time.perf_counter()
    loss, gM, gK, gP = run(Ms_T, K1_T, pulses, nsteps, True)
    torch.cuda.synchronize()
    wall = time.perf_counter() - w
    launches = eng.launch_count() - launches0
    # finite differences on a shorter trajectory
    fd_steps = args.adj_fd_steps
    loss2, gM2, gK2, gP2 = run(Ms_T, K1_T, pulses, fd_steps, True)
    h = args.adj_h
    rng = np.random.default_rng(11)
    errs, pairs = [], []
    for _ in range(args.adj_dirs):
        dM = Ms_T * rng.standard_normal(T)
        dK = 0.05 * rng.standard_normal(T)
        dP = np.abs(pulses).mean() * rng.standard_normal(pulses.shape)
        lp = run(Ms_T + h * dM, K1_T + h * dK, pulses + h * dP, fd_steps, False)
        lm = run(Ms_T - h * dM, K1_T - h * dK, pulses - h * dP, fd_steps, False)
        fd = (lp - lm) / (2 * h)
        ad = gM2 @ dM + gK2 @ dK + (gP2 * dP).sum()
        errs.append(abs(fd - ad) / max(abs(ad), 1e-30))
        pairs.append([float(fd), float(ad)])
    # the finite differences' own floor: a few ulps of the loss divided by 2h
    floor = 8.0 * np.finfo(np.float64).eps * abs(loss2) / (2.0 * h)
    resolvable = [k for k, (fd, ad) in enumerate(pairs) if abs(ad) * 1e-5 > floor]
    line = {"metric": "forward + adjoint wall time", "report": "adjoint", "value": wall, "unit": "s",
            "higher_is_better": False, "workload": WORKLOAD_NAMES[args.workload],
            "trajectory": {"steps": nsteps, "dt_ps": dt, "checkpoint_every": ckpt, "pulses": 20,
                           "steps_per_pulse": spp, "rhs_evals": 8 * nsteps, "vjp_evals": 4 * nsteps,
                           "note": "20 pulses span the trajectory (T/20 each; the configuration's 100 ps "
                                   "pulses would leave 18 of 20 beyond 2000 x 0.1 ps)"},
            "params": {"Ms_per_element": T, "K1_per_element": T, "pulse_amplitudes": 60},
            "loss": loss, "grad_norms": {"Ms": float(np.linalg.norm(gM)), "K1": float(np.linalg.norm(gK)),
                                         "pulses": float(np.linalg.norm(gP))},
            "sim_ps_per_s": nsteps * dt / wall,
            "forward_form": {"bem": args.adj_form, "cg": args.adj_cg}, "backward_cg": args.adj_bwd_cg,
            "poisson_rtol": args.adj_ksp,
            "fd_check": {"steps": fd_steps, "directions": len(errs), "h_rel": h, "fd_ad_pairs": pairs,
                         "max_rel_err": max(errs) if errs else None, "bound": 1e-5,
                         "fd_floor": floor,
                         "directions_resolvable": len(resolvable),
                         "max_rel_err_resolvable": max((errs[k] for k in resolvable), default=None),
                         "max_abs_err_over_max_derivative": (max(abs(a - b) for a, b in pairs)
                                                             / max(abs(b) for _, b in pairs)) if pairs else None,
                         "note": "a direction is resolvable when 1e-5 of its derivative exceeds the finite "
                                 "differences' floor (8 ulps of the loss over 2h); below it the relative error "
                                 "measures the floor, not the adjoint"},
            "gpu_launches": launches}
    print(json.dumps(line))


def run_jacobian_report(args):
    """The BDF's Newton matrix at each Jacobian level on the workload's
    chosen form: the reference's approximate Jacobian (exchange only), the
    local terms added, and the exact one (the demag response of every Krylov
    direction from its own Poisson solves at --jac-rtol).  Same relaxed start,
    same interval as the headline; device time, BDF / Newton / Krylov counts,
    and the final states' difference from the approximate Jacobian's."""
    import torch
    rank, world = dist_setup(1)
    torch.cuda.set_device(0)
    from nmag import _lib
    _lib.set_device(0)
    msh, base, seed = workload(args.workload)
    B = args.members
    anchor = args.anchor if args.form == "fp32x2" else 0.0
    start, relax_rec = relax_states(args, args.form, args.cg, B, msh, base, seed, anchor)
    out = {"report": "jacobian", "workload": WORKLOAD_NAMES[args.workload], "form": args.form, "cg": args.cg,
           "members": B, "interval_ps": args.steps * args.step_ps, "jacobian_demag_rtol": args.jac_rtol,
           "jv_at_level_0": args.jv,
           "relax": relax_rec, "levels": {}}
    ref_final = None
    for level in ("approximate", "local", "exact"):
        r = measure(args, args.form, args.cg, B, msh, start, world, 0, sample_clocks=False, anchor=anchor,
                    warmup=1, e2e=False, jacobian=level)
        row = {"value_ns_per_s": r["value"], "ms_per_step": r["ms_per_step"], "bdf_steps": r["bdf_steps"],
               "rhs_evals": r["rhs_evals"], "cg_iterations": r["cg_iterations"], "newton": r["newton"],
               "kernels_ms": {k: v["total_ms"] for k, v in r["kernels_ms"].items() if v["launches"]}}
        if ref_final is None:
            ref_final = r["m_final"]
        else:
            row["max_dm_final_vs_approximate"] = float(np.abs(r["m_final"] - ref_final).max())
        out["levels"][level] = row
        r["eng"].close()
        print(level, json.dumps(row), flush=True)
    print(json.dumps(out))


def particle_batch_config(n=256, seed=2):
    """The batching configuration: cubes with edge U[8, 40] nm at a 2 nm pitch
    (round(edge/2) cells per side), Ms U[4e5, 1.7e6] A/m, K1 U[0, 5e5] J/m^3
    along a random unit axis, alpha 0.1, field sweep direction random."""
    import nmag
    from nmag import SI, mesh
    rng = np.random.default_rng(seed)
    parts = []
    for k in range(n):
        c = int(round(rng.uniform(8.0, 40.0) / 2.0))
        msh = mesh.box_mesh(c, c, c, 2.0)
        Ms, K1 = rng.uniform(4e5, 1.7e6), rng.uniform(0.0, 5e5)
        ax = rng.standard_normal(3)
        ax /= np.linalg.norm(ax)
        hd = rng.standard_normal(3)
        hd /= np.linalg.norm(hd)
        mat = nmag.MagMaterial("p%d" % k, Ms=SI(Ms, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"), llg_damping=0.1,
                               llg_gamma_G=SI(2.211e5, "m/A s"),
                               anisotropy=nmag.uniaxial_anisotropy(axis=list(ax), K1=SI(K1, "J/m^3")))
        parts.append((msh.points, msh.simplices, mat.coefficients("nmag"), hd))
    return parts


def run_batch_report(args):
    """Batching form on the 256-particle configuration: setup, autotuned
    schedule, then timed CUDA-graph replays; reports the aggregate RHS and
    simulated-time throughput and the sweep's progress, and beside it the
    one-at-a-time RHS rate of a sample of particles on single handles (FP64
    BEM, same CG tolerance)."""
    import torch
    from nmag.batch import ParticleBatch
    from nmag import _lib
    torch.cuda.set_device(0)
    parts = particle_batch_config(args.particles)
    h_max = (1.0 / MU0) / 1e6   # 1 T / mu0 in simulation units
    w = time.perf_counter()
    # step tolerance 1e-7: the explicit integrator's |dm/dt| floor ~ tol/dt stays
    # well below the 1 deg/ns convergence threshold
    b = ParticleBatch(parts, n_stages=81, h_max=h_max, rtol=args.batch_tol, atol=args.batch_tol, cg_rtol=1e-6)
    setup = time.perf_counter() - w
    sizes = np.array(b.sizes)
    ms = [initial_m(n, (1.0, 1.0, 1.0), 100 + k) for k, n in enumerate(sizes)]
    # start along the first field so the sweep begins near saturation
    ms = [np.broadcast_to(np.asarray(parts[k][3]), (n, 3)) + 0.05 * ms[k] for k, n in enumerate(sizes)]
    ms = [m / np.linalg.norm(m, axis=1)[:, None] for m in ms]
    b.set_m(ms)
    w = time.perf_counter()
    threads, budget = b.autotune(trial_launches=2)
    tune = time.perf_counter() - w
    b.set_schedule(threads, budget)
    b.run(args.warmup)
    s0 = b.state()
    torch.cuda.synchronize()
    w = time.perf_counter()
    b.run(args.steps)
    torch.cuda.synchronize()
    wall = time.perf_counter() - w
    s1 = b.state()
    progress = None
    if args.batch_seconds > 0:   # keep sweeping for a wall-time budget and record the progress
        w2 = time.perf_counter()
        trace = []
        while time.perf_counter() - w2 < args.batch_seconds:
            b.run(args.steps)
            st = b.state()
            trace.append((round(time.perf_counter() - w2, 1), int(st["stage"].sum()), int(st["done"].sum())))
            if st["done"].all():
                break
        st = b.state()
        progress = {"wall_s": time.perf_counter() - w2, "stages_done": int(st["stage"].sum()),
                    "stages_total": 81 * len(sizes), "particles_done": int(st["done"].sum()),
                    "min_stage": int(st["stage"].min()), "median_stage": float(np.median(st["stage"])),
                    "trace_every": max(1, len(trace) // 12), "trace": trace[::max(1, len(trace) // 12)]}
    rhs = int((s1["rhs"] - s0["rhs"]).sum())
    node_rhs = float(((s1["rhs"] - s0["rhs"]) * sizes).sum())
    sim_ps = float((s1["t"] - s0["t"]).sum())
    # one-at-a-time reference: single handles on a size-stratified sample
    order = np.argsort(sizes)
    sample = order[np.linspace(0, len(order) - 1, 8).astype(int)]
    per_rhs = {}
    for k in sample:
        pts, sim, c_, hd = parts[k]
        mt = _lib.Material()
        mt.Ms, mt.exch_coeff, mt.C1, mt.C2, mt.C3 = c_["Ms"], c_["exch_coeff"], c_["C1"], c_["C2"], c_["C3"]
        mt.K1, mt.anis_coeff = c_["K1"], c_["anis_coeff"]
        for d in range(3):
            mt.axis[d] = c_["axis"][d]
        op = _lib.Options()
        op.do_demag = 1
        op.nbc_rtol = op.dbc_rtol = 1e-6
        op.nbc_atol = op.dbc_atol = 1e-50
        op.nbc_maxits = op.dbc_maxits = 10000
        op.bem_precision = 1   # FP32 BEM entries like the batch's blocks (like for like)
        eng = _lib.Engine(pts, sim, mt, op)
        eng.set_m(ms[k])
        eng.set_h_ext(np.broadcast_to(h_max * hd, (eng.N, 3)))
        dm = torch.tensor(ms[k].reshape(-1), device="cuda", dtype=torch.float64)
        out = torch.empty_like(dm)
        for _ in range(3):
            eng.rhs_device(dm.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(20):
            eng.rhs_device(dm.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        per_rhs[int(sizes[k])] = (time.perf_counter() - t0) / 20
        eng.close()
    xs = np.array(sorted(per_rhs))
    ys = np.array([per_rhs[x] for x in xs])
    est = float(np.interp(sizes, xs, ys).sum())   # seconds for one RHS of every particle, one at a time
    batch_rhs_rate = rhs / wall
    line = {"metric": "particle RHS evals/s (aggregate)", "report": "batch", "value": batch_rhs_rate,
            "unit": "RHS/s", "higher_is_better": True, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "data": "synthetic",
            "config": {"workload": "%d cubes, edge U[8,40] nm (seed 2), 2 nm pitch, nodes %d..%d (total %d), "
                                   "81-field +-1 T sweep, alpha 0.1" % (len(sizes), sizes.min(), sizes.max(),
                                                                         sizes.sum()),
                       "integrator": "Bogacki-Shampine 3(2), rtol = atol = %g, per particle" % args.batch_tol,
                       "bem": "FP32 blocks, FP64 row sums", "cg_rtol": 1e-6},
            "wall_s": wall, "setup_s": setup, "autotune_s": tune,
            "schedule": {"threads": threads, "budget": budget, "launches_per_graph": args.steps},
            "node_rhs_per_s": node_rhs / wall, "simulated_ps_per_s_aggregate": sim_ps / wall,
            "accepted_steps": int((s1["steps"] - s0["steps"]).sum()),
            "sweep": {"stages_done_total": int(s1["stage"].sum()), "stages_total": 81 * len(sizes),
                      "particles_done": int(s1["done"].sum())},
            "one_at_a_time": {"sample_sizes": [int(x) for x in xs], "rhs_s": [float(y) for y in ys],
                              "rhs_per_s_estimate": len(sizes) / est,
                              "note": "single handles (FP32 BEM entries and the same CG tolerance as the batch, "
                                      "one launch sequence per RHS), interpolated over the particle sizes"},
            "speedup_vs_one_at_a_time": batch_rhs_rate / (len(sizes) / est),
            "sweep_run": progress}
    print(json.dumps(line))
    b.close()


def run_ours(args):
    import torch
    rank, world = dist_setup(args.gpus)
    local = int(os.environ.get("LOCAL_RANK_DEVICE", os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(local)
    torch.cuda.init()
    from nmag import _lib
    _lib.set_device(local)
    msh, base, seed = workload(args.workload)
    B = args.members
    anchor = args.anchor if args.form == "fp32x2" else 0.0
    # one relaxation for both forms (untimed setup): the ensemble's members
    # from seeds seed..seed+B-1; the plain film starts from member 0's state
    start, relax_rec = relax_states(args, args.form, args.cg, B, msh, base, seed, anchor)
    r = measure(args, args.form, args.cg, B, msh, start, world, local, anchor=anchor)
    plain = None
    if args.compare and not (args.form == "fp64" and args.cg == "fp64" and B == 1):
        start0 = start[0] if B > 1 else start
        plain = measure(args, "fp64", "fp64", 1, msh, start0, world, local, sample_clocks=False,
                        warmup=1, e2e=False, jv="fp64")
    if rank != 0:
        return
    line = {
        "metric": "simulated ns/wall-s", "value": r["value"], "unit": "ns/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": {"fp64": "f64", "fp32": "f32 matrix, f64 sums",
                  "fp32x2": "f32+bf16 matrix, compensated f32 products (~2^-44)" + (
                      "; anchored: f32 products of the drift from the last compensated product"
                      if anchor > 0 else "")}[args.form] + (
                      "; f32 Jacobian-vector products" if args.jv == "fp32" else ""),
        "data": "synthetic",
        "config": config_dict(args, msh),
        "rhs_evals_per_s": r["rhs_evals_per_s"], "bdf_steps": r["bdf_steps"], "rhs_evals": r["rhs_evals"],
        "wall_value_s": r["wall_value_s"],
        "roofline": r["roofline"],
        "dominant_kernel": r["dominant_kernel"],
        "kernels_ms": r["kernels_ms"],
        "cg_iterations": r["cg_iterations"],
        "relax": relax_rec,
        "per_member_value": r["value"] / B,
        "e2e": {"value": r["e2e"], "unit": "ns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": r["d2h"],
                "call": "nmag.Simulation.advance_time + get_subfield_average_siv('m'), same interval and start "
                        "state as value"},
        "avg_m_final": [float(v) for v in r["trace"][-1]],
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
    }
    if r["anchored"] is not None:
        line["anchored"] = r["anchored"]
    if plain is not None:
        line["plain_fp64"] = {"value": plain["value"], "e2e": plain["e2e"], "ms_per_step": plain["ms_per_step"],
                              "rhs_evals_per_s": plain["rhs_evals_per_s"], "bdf_steps": plain["bdf_steps"],
                              "roofline": plain["roofline"], "kernels_ms": plain["kernels_ms"],
                              "gpu_launches": plain["launches"]}
        line["speedup_vs_plain_fp64"] = r["value"] / plain["value"]
        line["heff_rel_err_vs_fp64"] = heff_error(args, r, msh)
        # member 0 starts from the plain run's state: <m> at every record of the interval
        line["avg_m_diff_vs_plain_fp64"] = float(np.abs(r["trace"] - plain["trace"]).max())
    if anchor > 0:
        err, prod, nref, nev = anchor_path_error(args, r, msh)
        line["anchored"]["path_error"] = {"heff_rel_err_vs_fp64": err, "products": prod, "refreshes": nref,
                                          "evaluations": nev,
                                          "windows": "records %s (ps): consecutive states of the e2e leg, 4 blends "
                                                     "per 1 ps record interval" % (WINDOW_RECORDS,)}
        line["heff_rel_err_vs_fp64"] = max(line.get("heff_rel_err_vs_fp64", 0.0), err)
    if world == 1 and not args.no_cpu_baseline:
        cr = cpu_reference_run(args, msh, base, seed, steps=args.cpu_records, warmup=0, max_wall=20.0)
        cpu_value = (cr["sim_ps"] * 1e-3) / cr["wall_s"]
        line["cpu_baseline"] = {"value": cpu_value, "unit": "ns/s", "cores": cr["cores"],
                                "kind": "port",
                                "sample": "%d x %.2f ps records of one film's dynamics on the CPU restatement, "
                                          "after a %g ps relax at alpha=1" % (cr["steps"], cr["dt"], args.relax_ps),
                                "rhs_evals_per_s": cr["nfe"] / cr["wall_s"]}
        if plain is not None:
            line["plain_fp64"]["vs_cpu_baseline"] = plain["value"] / cpu_value
            line["plain_fp64"]["rhs_evals_per_s_vs_cpu_baseline"] = (plain["rhs_evals_per_s"]
                                                                     / line["cpu_baseline"]["rhs_evals_per_s"])
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="fp32x2", choices=["fp64", "fp32", "fp32x2", "bf16x3"],
                    help="BEM product: fp64; fp32 (FP32 entries, FP64 sums); fp32x2 (FP32 + BF16 residual "
                         "entries, compensated FP32 products); bf16x3 (three BF16 planes, tensor cores)")
    ap.add_argument("--precision-members", type=int, default=0,
                    help="--report precision: fields per ensemble (0: 128 for bf16x3, else 8)")
    ap.add_argument("--workload", default="film", choices=["film", "cube", "film_small"])
    ap.add_argument("--step-ps", type=float, default=50.0,
                    help="simulated time per step (20 steps: the configured 1 ns)")
    ap.add_argument("--record-ps", type=float, default=1.0, help="<m> is read every record_ps")
    ap.add_argument("--relax-cap-ps", type=float, default=5000.0,
                    help="cap of the simulated time of the (untimed) relaxation to 1 deg/ns")
    ap.add_argument("--relax-ps", type=float, default=10.0,
                    help="the CPU arms' truncated relax at alpha=1 before their sampled records")
    ap.add_argument("--cpu-records", type=int, default=20,
                    help="records of the CPU baseline sample in our line (bounded by 20 s of CPU work)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cg", default="fp32", choices=["fp64", "fp32"],
                    help="Poisson CG: FP64, or FP32 iterations with FP64 residual refinement")
    ap.add_argument("--anchor-product", default="fp32", choices=["fp32", "fp16"],
                    help="difference product of the anchored ensemble form: FP32 matrix copy or FP16 copy "
                         "in tensor-core fragment order")
    ap.add_argument("--cg-sweeps", type=int, default=0,
                    help="FP32 inner CG: damped Jacobi sweeps on each block's rows in the preconditioner")
    ap.add_argument("--anchor", type=float, default=1e-2,
                    help="fp32x2: anchored product tolerance (B x = B x0 + B32 (x - x0) while the max-norm drift "
                         "of x from x0 stays below it; 0 = off)")
    ap.add_argument("--members", type=int, default=8,
                    help="ensemble size: B films on the one mesh integrated together (value summed over members)")
    ap.add_argument("--adj-steps", type=int, default=2000)
    ap.add_argument("--adj-fd-steps", type=int, default=100)
    ap.add_argument("--adj-dirs", type=int, default=32)
    ap.add_argument("--adj-h", type=float, default=1e-6, help="relative step of the central differences")
    ap.add_argument("--adj-ksp", type=float, default=1e-12,
                    help="Poisson solves' rtol in the differentiation report (the finite differences at "
                         "h = 1e-6 need the loss accurate well beyond 1e-6 relative)")
    ap.add_argument("--adj-form", default="fp32x2", choices=["fp64", "fp32x2"],
                    help="BEM product of the RK4 forward pass (the adjoint's B^T product is FP64)")
    ap.add_argument("--adj-cg", default="fp64", choices=["fp64", "fp32"],
                    help="Poisson CG of the RK4 forward pass")
    ap.add_argument("--adj-bwd-cg", default="fp32", choices=["fp64", "fp32"],
                    help="Poisson CG of the adjoint's backward pass (fp32: FP64-refined to the same tolerance)")
    ap.add_argument("--particles", type=int, default=256)
    ap.add_argument("--batch-tol", type=float, default=1e-7)
    ap.add_argument("--batch-seconds", type=float, default=0.0,
                    help="after the timed launches, keep sweeping for this wall time and report the progress")
    ap.add_argument("--rhs", type=int, default=128, help="--report bem: right-hand sides per product")
    ap.add_argument("--cg-no-coarse", action="store_true",
                    help="Neumann CG with Jacobi alone (no aggregation coarse level)")
    ap.add_argument("--poisson-rtol", type=float, default=None,
                    help="relative tolerance of the Neumann and Dirichlet solves in every leg (default: the "
                         "reference's 1e-5)")
    ap.add_argument("--jv", default="fp32", choices=["fp64", "fp32"],
                    help="arithmetic of the BDF's Jacobian-vector products and block preconditioner "
                         "(the chosen form; the plain FP64 comparison always uses fp64)")
    ap.add_argument("--jac-rtol", type=float, default=1e-3,
                    help="Poisson tolerance of the exact Jacobian's demag response (--report jacobian)")
    ap.add_argument("--report", default=None, choices=["precision", "adjoint", "batch", "bem", "jacobian"],
                    help="precision: H_eff / energy error of the FP32 form against FP64 over --fields random fields")
    ap.add_argument("--fields", type=int, default=1000)
    ap.add_argument("--no-compare", dest="compare", action="store_false",
                    help="skip the plain FP64 single-film run reported beside the chosen form")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.report == "precision":
        run_precision_report(args)
    elif args.report == "adjoint":
        run_adjoint_report(args)
    elif args.report == "bem":
        run_bem_report(args)
    elif args.report == "batch":
        run_batch_report(args)
    elif args.report == "jacobian":
        run_jacobian_report(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
