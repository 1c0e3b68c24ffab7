"""Benchmark: simulated ns per wall-second of nmag's LLG path on the film.

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
                       [--form fp64|fp32] [--workload film|cube]
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

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "nmag-src_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

MU0 = 4e-7 * np.pi
H_EXT_MT = (-24.6, 4.3, 0.0)

# DRAM bytes per launch of the BEM product divided by its algorithmic bytes,
# from one ncu capture on the 8,562-boundary-node profiling film (matrix
# 586.6 MB > L2; profiles/k_gemv_f64_film_small.txt: 590.04 MB read+written).
# The traffic grows with the matrix entries, so it scales to the full film.
NCU_TRAFFIC_RATIO = {"fp64": (586.81 + 3.23) / 586.60}


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
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_reference_run(args, msh, base, seed, steps, warmup, max_wall=25.0, sample_ps=None):
    """Time the oracle (CPU restatement, all host threads) on the workload:
    the same relax stage (alpha = 1, no field, RELAX_PS), then the timed
    alpha = 0.02 dynamics under H_ext."""
    import oracle
    t0 = time.perf_counter()
    om = oracle.OracleMesh(msh.points, msh.simplices, nthreads=0)
    m = initial_m(msh.n_nodes, base, seed)
    if args.relax_ps > 0:
        r = oracle.OracleSim(om, material(1.0).coefficients("nmag"))
        r.ts_init(m, rtol=1e-6, atol=1e-6)
        _, m = r.ts_advance(args.relax_ps)
        del r
    s = oracle.OracleSim(om, material(0.02).coefficients("nmag"))
    s.set_h_ext(h_ext_su())
    s.ts_init(m, rtol=1e-6, atol=1e-6)
    setup = time.perf_counter() - t0
    t = 0.0
    dt = sample_ps or args.step_ps
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
            "cores": os.cpu_count()}


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
                         "sample": "%d x %.2f ps of the workload on the CPU restatement (oracle/, OpenMP)"
                                   % (r["steps"], args.step_ps)},
        "e2e": {"value": value, "unit": "ns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own build (OCaml/Python 2/PETSc/SUNDIALS) cannot run here; this arm times "
                "the CPU restatement of its algorithms",
    }
    print(json.dumps(line))


WORKLOAD_NAMES = {
    "film": "film 500x125x3 nm, 30753 nodes, 21002 boundary nodes, alpha 0.02, H_ext (-24.6,4.3,0) mT",
    "cube": "cube 30 nm, 1331 nodes, 602 boundary nodes",
    "film_small": "film 250x100x3 nm (profiling size), 12423 nodes, 8562 boundary nodes, alpha 0.02",
}


def config_dict(args, msh):
    return {"workload": WORKLOAD_NAMES[args.workload],
            "relax": "alpha=1, H_ext=0 for %.3g ps before the timed dynamics (untimed)" % args.relax_ps,
            "nodes": int(msh.n_nodes), "tets": int(msh.n_tets), "step": "%.3g ps advance + <m> read" % args.step_ps,
            "form": args.form, "cg": args.cg, "members": args.members,
            "rtol": 1e-6, "atol": 1e-6, "max_order": 2, "krylov_max": 300,
            "l2": "BEM matrix (nb^2 x %d B) larger than L2; no explicit flush" % (8 if args.form == "fp64" else 4)}


def run_ours(args):
    import torch
    import nmag
    from nmag import SI
    rank, world = dist_setup(args.gpus)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    torch.cuda.init()
    msh, base, seed = workload(args.workload)
    B = args.members
    # fp32 form: FP32 BEM matrix (FP64 sums); --cg fp32: FP32 CG iterations with FP64 residual refinement
    sim = nmag.Simulation("bench", bem_precision=args.form, cg_precision=args.cg, n_members=B)
    sim.load_mesh(msh, [("film", material(0.02))], unit_length=SI(1e-9, "m"))
    eng = sim.engine
    if B > 1:   # member b starts from the workload's initial state with seed + b
        sim.set_m(np.stack([initial_m(msh.n_nodes, base, seed + b) for b in range(B)]))
    else:
        sim.set_m(initial_m(msh.n_nodes, base, seed))
    relax_wall = 0.0
    if args.relax_ps > 0:   # relax stage: alpha = 1, no applied field
        w = time.perf_counter()
        sim.set_damping(1.0)
        sim.reinitialise(initial_time=0)
        sim.advance_time(SI(args.relax_ps * 1e-12, "s"))
        sim.set_damping(0.02)
        relax_wall = time.perf_counter() - w
    sim.set_H_ext(h_ext_su() * 1e6, SI(1.0, "A/m"))
    sim.reinitialise(initial_time=0)
    ps = args.step_ps
    t = 0.0
    for _ in range(args.warmup):
        t += ps
        eng.ts_advance(t)
    # ---- timed region: device-resident value leg ----
    sampler = ClockSampler(local)
    sampler.start()
    eng.profile(True)
    launches0 = eng.launch_count()
    cg0 = eng.cg_iterations()
    _, st0 = eng.ts_advance(t)   # no-op advance to read the counters
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    dev_ms = 0.0
    w0 = time.perf_counter()
    avgs = []
    for _ in range(args.steps):
        t += ps
        _, st = eng.ts_advance(t)
        dev_ms += float(eng.timings()[0])
        avgs.append(eng.averages())
    torch.cuda.synchronize()
    wall_value = time.perf_counter() - w0
    barrier(world)
    launches = eng.launch_count() - launches0
    cg1 = eng.cg_iterations()
    eng.profile(False)
    prof = eng.profile_read()
    clocks = sampler.stop()
    nfe = st["nfe"] - st0["nfe"]
    nst = st["nst"] - st0["nst"]
    # ---- e2e leg through the public API (advance_time copies m to the host) ----
    sim.clock.stage_time_su = t
    sim._last_nst = st["nst"]
    torch.cuda.synchronize()
    barrier(world)
    w1 = time.perf_counter()
    for _ in range(args.steps):
        t += ps
        sim.advance_time(SI(t * 1e-12, "s"))
        sim.get_subfield_average_siv("m")
    torch.cuda.synchronize()
    wall_e2e = time.perf_counter() - w1
    dev_s = max_over_ranks(dev_ms * 1e-3, world)
    wall_e2e = max_over_ranks(wall_e2e, world)
    sim_ns_total = world * B * args.steps * ps * 1e-3   # summed over ensemble members
    value = sim_ns_total / dev_s
    e2e_value = sim_ns_total / wall_e2e
    if rank != 0:
        return
    nb = eng.nb
    gl, gms = prof["bem_gemv"]
    elem = 8 if args.form == "fp64" else 4
    nm = min(B, 8)   # members per BEM launch
    bytes_per_launch = nb * nb * elem + 2 * nm * nb * 8
    hbm, peak_kind = peaks()
    roof = None
    if gl > 0:
        avg_ms = gms / gl
        achieved = bytes_per_launch / (avg_ms * 1e-3) / 1e9
        kname = ("k_gemv_" if B == 1 else "k_gemm_") + ("f64" if args.form == "fp64" else "f32")
        roof = {"bound": "hbm" if not (B > 1 and args.form == "fp64") else "fp64 pipe (bytes shown)",
                "kernel": kname,
                "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "peak_kind": peak_kind,
                "traffic": (NCU_TRAFFIC_RATIO[args.form] * bytes_per_launch / 1e9
                            if args.form in NCU_TRAFFIC_RATIO else None),
                "traffic_unit": "GB per launch (ncu dram__bytes_read+write, scaled from the profiling film)",
                "launches": gl, "avg_launch_ms": avg_ms,
                "algorithmic_bytes_per_launch": bytes_per_launch,
                "share_of_step": gms / max(dev_ms, 1e-9)}
    line = {
        "metric": "simulated ns/wall-s", "value": value, "unit": "ns/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_s * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(args, msh),
        "rhs_evals_per_s": nfe / dev_s * world, "bdf_steps": nst, "rhs_evals": nfe,
        "wall_value_s": wall_value,
        "roofline": roof,
        "kernels_ms": {k: {"launches": v[0], "total_ms": v[1]} for k, v in prof.items()},
        "cg_iterations": {"neumann": cg1[0] - cg0[0], "dirichlet": cg1[1] - cg0[1]},
        "relax_wall_s": relax_wall,
        "e2e": {"value": e2e_value, "unit": "ns/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": B * msh.n_nodes * 3 * 8 + 24,
                "call": "nmag.Simulation.advance_time + get_subfield_average_siv('m')"},
        "gpu_launches": launches,
        "clocks": clocks,
        "avg_m_last": [float(x) for x in avgs[-1]] if avgs else None,
    }
    if world == 1 and not args.no_cpu_baseline:
        r = cpu_reference_run(args, msh, base, seed, steps=2, warmup=0, max_wall=20.0, sample_ps=0.5 * ps)
        line["cpu_baseline"] = {"value": (r["sim_ps"] * 1e-3) / r["wall_s"], "unit": "ns/s", "cores": r["cores"],
                                "kind": "port",
                                "sample": "%d x %.2f ps from the seeded initial state on the CPU restatement"
                                          % (r["steps"], 0.5 * ps),
                                "rhs_evals_per_s": r["nfe"] / r["wall_s"]}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--workload", default="film", choices=["film", "cube", "film_small"])
    ap.add_argument("--step-ps", type=float, default=1.0)
    ap.add_argument("--relax-ps", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cg", default="fp64", choices=["fp64", "fp32"],
                    help="Poisson CG: FP64, or FP32 iterations with FP64 residual refinement")
    ap.add_argument("--members", type=int, default=1,
                    help="ensemble size: B films on the one mesh integrated together (value summed over members)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
