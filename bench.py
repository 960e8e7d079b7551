#!/usr/bin/env python3
"""Benchmark of the fermion-matrix hot path on GB300.

Workload (the reference's second configuration): Wilson-clover fermion on a
32^4 lattice, gauge links exp(i*0.3*H) with H Hermitian traceless and
complex-Gaussian entries (seeded), mass 0.05, csw_r = csw_t = 1.0, boundary
phases [1,1,1,-1], one complex-Gaussian source.  Synthetic data (there is no
dataset involved).

One step = one propagator solve to true FP64 residual 1e-10 with
defect_correcting(mixed_precision(preconditioned(eo2_ne, cg(1e-5)), single,
double), eps=1e-10) -- the mixed method.  `value` = mixed solves/s with the
source resident in HBM; `e2e` = the same through the public API from pinned
host memory (source H2D and solution D2H inside the timed region).  The plain
FP64 eo2_ne CG (eps 1e-10) is measured beside it.  Inputs (gauge field
604 MB, clover 1.2 GB, source 201 MB FP64) are larger than the 129 MB L2, so
no L2 flush is needed between steps.

--impl reference runs the CPU restatement of the same solve (the reference's
Grid CPU operator cannot be built here) on all host cores: each step is one
full mixed solve, timed.

After the timed region the default line also carries compact measurements
of the other configurations (c1, c3, c4, c5, each with the FP64 oracle
residual of its solves), the reference's own Dslash benchmark and the rows
beyond the hot path; the figures to read (mixed, plain, their ratio) come
last in the line.
"""
import argparse
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Dslash HBM GB/s; CG solves/s at FP64 residual 1e-10 (mixed vs plain); p99 ms"
CFG = dict(dims=[32, 32, 32, 32], gauge_eps=0.3, gauge_seed=2024, src_seed=7, mass=0.05, csw=1.0,
           phases=[1.0, 1.0, 1.0, -1.0], tol=1e-10, inner_tol=1e-5)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbf", choices=["gbf", "reference"])
    ap.add_argument("--dims", type=str, default=None, help="override lattice, e.g. 16,16,16,16 (tests only)")
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-next-rows", action="store_true",
                    help="c2: skip the measurements of the rows beyond the hot path after the timed region")
    ap.add_argument("--no-configs", action="store_true",
                    help="c2: skip the compact c1, c3, c4 and c5 measurements after the timed region")
    ap.add_argument("--no-dhop-benchmark", action="store_true",
                    help="c2: skip the reference's Dslash benchmark (Mobius Dhop 64.32.32.32 Ls 12) after the timed region")
    ap.add_argument("--profile-dslash", action="store_true",
                    help="profiling case: one operator only, one eo2_ne CG of 12 iterations")
    ap.add_argument("--profile-precision", default="single", choices=["single", "double", "double_float", "half"],
                    help="precision of the --profile-dslash operator")
    ap.add_argument("--profile-next", action="store_true",
                    help="profiling case of the kernels beyond the hot path: mode matrix, chiral shift, slice copy, "
                         "multi-shift update, block-CG Gram and linear combination (a few GB on the device)")
    ap.add_argument("--profile-dhop", action="store_true",
                    help="profiling case: the reference's Dhop benchmark on --dims (default 64,32,32,8), Ls 12, "
                         "--profile-precision only, 20 applications")
    ap.add_argument("--profile-mobius", action="store_true",
                    help="profiling case: FP32 mobius 12^3x24 Ls 12 with 12 packed rhs, 12 CG iterations")
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "next", "dslash"],
                    help="c2 (default): wilson_clover 32^4 mixed vs plain; c1: wilson_clover 8^4; c3: mobius "
                         "16^3x32 Ls=12, 12 point sources; c4: mobius 32^3x64 Ls=16, 12 sources; c5: serving stream; "
                         "next: the solver layers, operators and IO beyond the hot path; dslash: the reference's "
                         "Dslash benchmark (Mobius Dhop, 64.32.32.32, Ls 12)")
    ap.add_argument("--requests", type=int, default=40, help="c5: number of requests")
    ap.add_argument("--inner", default="single", choices=["single", "half"], help="c3/c4 inner precision")
    ap.add_argument("--rhs-group", type=int, default=0, help="c4: right-hand sides solved together (0: auto)")
    ap.add_argument("--with-plain", action="store_true",
                    help="c3: also time one plain FP64 and one plain double-float packed solve of the same sources")
    ap.add_argument("--cg-graph", type=int, default=0,
                    help="c2: CG iterations per CUDA graph with a host convergence check between graphs (0: the "
                         "library default, 16; -1: the whole CG loop on the device, one graph with a conditional "
                         "while node; -2: no graphs, every kernel launched from the host, for per-kernel launch "
                         "lists under ncu)")
    ap.add_argument("--solver", default="cg", choices=["cg", "block_cg"],
                    help="c3/c4 inner solver: independent CG per packed rhs, or block CG over them")
    return ap.parse_args()


def max_over_ranks(ms, dist=None, device="cpu"):
    """Max of a per-rank duration over all ranks (the whole job is as slow as
    its slowest replica)."""
    import torch

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    if dist is not None and dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, steps, max_ms):
    """Units processed by all ranks per second: replicas, weak scaling."""
    return world * steps / (max_ms / 1000.0)


def run_profile_mobius(args):
    """Profiling case of the 5D multi-rhs path (about 4 GB on the device)."""
    import torch

    import gpt_gb300 as g

    g.load()
    dims = [12, 12, 12, 24]
    grid = g.grid(dims, g.double)
    U = g.qcd.gauge.random_su3_device(grid, 0.4, 4242)
    params = dict(Ls=12, b=1.5, c=0.5, M5=1.8, mass_plus=0.01, mass_minus=0.01, boundary_phases=[1.0, 1.0, 1.0, -1.0],
                  n_rhs=12)
    op = g.qcd.fermion.mobius_operator(U, params, precision=g.single)
    src = op.F_lattice()
    L = g._lib.load()
    V = grid.gsites
    nat = torch.empty(V * 12 * 24, dtype=torch.float64, device="cuda")
    for k in range(12):
        g._lib.check(L.gbf_random_spinor(V * 12 * 12, 50 + k, nat.data_ptr(), g.core.stream_ptr()))
        g._lib.check(L.gbf_field_import(src.layout.op, nat.data_ptr(), src.ptr, k, 1, g.core.stream_ptr()))
    x = op.F_lattice()
    for _ in range(args.warmup):
        op._solve_eo2ne_cg(x, src, 1e-30, 12)
    r = op._solve_eo2ne_cg(x, src, 1e-30, 12, 0, 1)
    torch.cuda.synchronize()
    out = {"profile_case": "mobius FP32 12^3x24 Ls 12, 12 rhs, eo2_ne CG 12 iterations", "iterations": r.iterations,
           "kernel_ms": list(r.kernel_ms), "kernel_launches": list(r.kernel_launches)}
    if args.solver == "block_cg":
        rb = op._solve_eo2ne_block_cg(x, src, 1e-30, 4)
        torch.cuda.synchronize()
        out["block_cg_iterations"] = rb.iterations
    print(json.dumps(out))
    return 0


def _common_line(metric, value, unit, args, world, total_ms, dims_cfg, dtype, extra):
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic", "config": dims_cfg}
    line.update(extra)
    return line


def measure_mobius(which, warmup, steps, inner="single", solver_kind="cg", rhs_group=0, with_plain=False,
                   max_groups=None, oracle_residual=True):
    """c3: Mobius 16^3x32, Ls 12, b 1.5, c 0.5, M5 1.8, mass 0.01, gauge eps 0.4,
    12 point sources (every spin-colour component at site 0) as one packed
    12-rhs field, propagator = Export * solve * Import, to true residual 1e-8.
    c4: Mobius 32^3x64, Ls 16, mass 0.005, 12 Gaussian sources, to 1e-10,
    solved in groups of right-hand sides that fit HBM (max_groups limits how
    many groups one step solves).  With oracle_residual the FP64 oracle's
    true residual |b - M x| / |b| of every 5D system of the last step is
    computed on the host.  Returns (summary dict, total ms, config dict)."""
    import torch

    import gpt_gb300 as g

    L = g.load()
    if which == "c3":
        dims, Ls, mass, geps, tol, nsrc = [16, 16, 16, 32], 12, 0.01, 0.4, 1e-8, 12
        group = 12
    else:
        dims, Ls, mass, geps, tol, nsrc = [32, 32, 32, 64], 16, 0.005, 0.4, 1e-10, 12
        group = rhs_group
    grid = g.grid(dims, g.double)
    U = g.qcd.gauge.random_su3_device(grid, geps, 4242)
    inner_prec = g.half if inner == "half" else g.single
    rhs_tuning = None
    if not group:
        # RHS block size by the autotuner: time 3 inner CG iterations of the
        # packed inner operator per candidate that fits (the outer FP64 loop
        # needs about as much memory again: budget half the free memory)
        from gpt_gb300 import tune as _tune

        base = dict(Ls=Ls, b=1.5, c=0.5, M5=1.8, mass_plus=mass, mass_minus=mass, boundary_phases=[1.0, 1.0, 1.0, -1.0])
        free, _ = torch.cuda.mem_get_info()
        # whole mixed solve per rhs: about 8 FP64 and 7 FP32 full 5D fields
        per_rhs = 8 * 192 * grid.gsites * Ls + 7 * 96 * grid.gsites * Ls
        cands = [k for k in (1, 2, 3, 4, 6) if k * per_rhs <= 0.85 * free]
        rhs_tuning = _tune.rhs_group(
            lambda k: g.qcd.fermion.mobius_operator(U, dict(base, n_rhs=k), precision=inner_prec), nsrc,
            candidates=cands, budget_bytes=int(0.85 * free))
        group = rhs_tuning["params"][0]
        gc.collect()
        torch.cuda.empty_cache()
    inner_tol = 1e-5 if inner == "single" else 3e-3
    V = grid.gsites
    ngroups = (nsrc + group - 1) // group
    if max_groups:
        ngroups = min(ngroups, max_groups)
    nsolved = min(nsrc, ngroups * group)
    params = dict(Ls=Ls, b=1.5, c=0.5, M5=1.8, mass=mass, boundary_phases=[1.0, 1.0, 1.0, -1.0], n_rhs=group)
    op = g.qcd.fermion.mobius(U, params)
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    inner_kind = inv.block_cg if solver_kind == "block_cg" else inv.cg
    inner_cg = inner_kind({"eps": inner_tol, "maxiter": 50000})
    dc = inv.defect_correcting(inv.mixed_precision(inv.preconditioned(pc.eo2_ne(), inner_cg), inner_prec, g.double),
                               eps=tol, maxiter=200)
    solver = dc(op)
    last5 = {}

    def prop(s4):
        # propagator = Export * solver * Import (operator/base.py:270-286)
        b5 = op.ImportPhysicalFermionSource(s4)
        x5 = solver(b5)
        last5.clear()  # keep only the latest group's 5D fields (HBM)
        last5[id(s4)] = (b5, x5)
        return op.ExportPhysicalFermionSolution(x5)

    srcs = []
    for grp in range(ngroups):
        s4 = op.U_lattice()
        nat = torch.zeros(V * 24, dtype=torch.float64, device="cuda")
        for k in range(group):
            kk = grp * group + k
            if which == "c3":
                nat.zero_()
                nat[2 * kk] = 1.0  # site 0, spin-colour component kk (real part)
            else:
                g._lib.check(L.gbf_random_spinor(V * 12, 1000 + kk, nat.data_ptr(), g.core.stream_ptr()))
            g._lib.check(L.gbf_field_import(s4.layout.op, nat.data_ptr(), s4.ptr, k, 0, g.core.stream_ptr()))
        srcs.append(s4)
    stream = torch.cuda.current_stream()

    def one_step():
        outs = []
        for s4 in srcs:
            outs.append(prop(s4))
        return outs

    for _ in range(warmup):
        one_step()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    torch.cuda.synchronize()
    n0 = L.gbf_launch_count()
    before = inner_cg.total_iterations
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        outs = one_step()
    e1.record(stream)
    torch.cuda.synchronize()
    n1 = L.gbf_launch_count()
    clk = clocks.stop()
    total_ms = e0.elapsed_time(e1)
    inner_its = (inner_cg.total_iterations - before) // max(1, steps)
    # device memory in use with the operators, Krylov workspace and the last
    # group's fields resident: every live allocation on the GPU, torch's and
    # the library's, as total - free after torch's cache of freed blocks is
    # released; beside it the peak of torch's live tensors
    gc.collect()
    torch.cuda.empty_cache()
    free_b, total_b = torch.cuda.mem_get_info()
    used_gb = (total_b - free_b) / 1e9
    torch_peak_gb = torch.cuda.max_memory_allocated() / 1e9
    # true residual of the 5D systems of the last group, FP64 on the device
    worst = 0.0
    for b5, x5 in last5.values():
        r5 = op.F_lattice()
        op.M(r5, x5)
        g.axpby(r5, -1.0, r5, 1.0, b5)
        nr, nb = g.norm2(r5), g.norm2(b5)
        nr, nb = ([nr], [nb]) if group == 1 else (nr, nb)
        worst = max(worst, max(math.sqrt(a / b) for a, b in zip(nr, nb)))
    # and with the FP64 oracle on the host, every rhs of the last group
    oracle_res = None
    if oracle_residual:
        import oracle as o

        ref = o.mobius(U.host(), dims, Ls=Ls, b=1.5, c=0.5, M5=1.8, mass=mass, boundary_phases=[1, 1, 1, -1])
        oracle_res = []
        for b5, x5 in last5.values():
            for k in range(group):
                xb, bb = x5.get_natural(k), b5.get_natural(k)
                rr = bb - ref.apply("M", xb)
                oracle_res.append(math.sqrt(o.norm2(rr) / o.norm2(bb)))
                del xb, bb, rr
        del ref
    value = nsolved * steps / (total_ms / 1000.0)
    plain = {}
    if with_plain and ngroups == 1:
        # the same packed sources with the plain method: eo2_ne CG in FP64
        # and in double-float, to the same true residual
        for name, pop in [("plain_fp64", op), ("plain_double_float", op.converted(g.double_float))]:
            # eps on the eo2_ne normal residual; tol / 10 makes the true 5D
            # residual of M x = b reach tol (measured ratio about 6)
            pcg = inv.cg({"eps": tol / 10, "maxiter": 50000})
            psolve = inv.preconditioned(pc.eo2_ne(), pcg)(pop)
            s4 = srcs[0]
            if pop is not op:
                s4c = pop.U_lattice()
                g.convert(s4c, s4)
                s4 = s4c
            b5 = pop.ImportPhysicalFermionSource(s4)
            torch.cuda.synchronize()
            q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            q0.record(stream)
            x5 = psolve(b5)
            pop.ExportPhysicalFermionSolution(x5)
            q1.record(stream)
            torch.cuda.synchronize()
            ms = q0.elapsed_time(q1)
            xr = op.F_lattice()
            g.convert(xr, x5)
            b5r = op.F_lattice()
            g.convert(b5r, b5)
            r5 = op.F_lattice()
            op.M(r5, xr)
            g.axpby(r5, -1.0, r5, 1.0, b5r)
            nr, nb = g.norm2(r5), g.norm2(b5r)
            nr, nb = ([nr], [nb]) if group == 1 else (nr, nb)
            plain[name] = {"solves_per_s": nsolved / (ms / 1000.0), "ms_per_step": ms, "cg_iterations": pcg.last.iterations,
                           "true_residual_5d": max(math.sqrt(a / b) for a, b in zip(nr, nb))}
            del psolve, x5, b5, xr, b5r, r5
        plain["mixed_over_plain_fp64"] = value / plain["plain_fp64"]["solves_per_s"]
        plain["mixed_over_plain_double_float"] = value / plain["plain_double_float"]["solves_per_s"]
    cfg = {"workload": f"mobius {'x'.join(map(str, dims))} Ls {Ls} b 1.5 c 0.5 M5 1.8 mass {mass} gauge eps {geps}, "
                       f"{nsolved} {'point' if which == 'c3' else 'gaussian'} sources in {ngroups} packed group(s) of "
                       f"{group}, propagator Export*solve*Import, defect correction ({inner} inner {solver_kind}, tol "
                       f"{inner_tol}) to true residual {tol}", "lattice": dims, "Ls": Ls,
           "l2_policy": "inputs larger than L2; no flush", "parallelism": "replicas"}
    r = {"solves_per_s": value, "ms_per_solve": total_ms / steps / nsolved, "sources_per_step": nsolved,
         "packed_group": group, "inner": inner, "solver": solver_kind,
         "true_residual_5d": worst, "true_residual_oracle_max": max(oracle_res) if oracle_res else None,
         "true_residual_oracle": oracle_res,
         "inner_cg_iterations_per_step": inner_its, "outer_corrections": len(dc.history) - 1,
         "device_memory_used_gb": used_gb, "device_memory_total_gb": total_b / 1e9,
         "torch_peak_allocated_gb": torch_peak_gb, "gpu_launches": int(n1 - n0), "clocks": clk, **plain,
         **({"rhs_group_tuning": rhs_tuning["results"]} if rhs_tuning else {})}
    return r, total_ms, cfg


def run_mobius_config(args, which):
    r, total_ms, cfg = measure_mobius(which, args.warmup, args.steps, args.inner, args.solver, args.rhs_group,
                                      args.with_plain)
    line = _common_line(METRIC, r["solves_per_s"], "solves/s", args, 1, total_ms, cfg,
                        f"{'f16' if args.inner == 'half' else 'f32'} inner / f64 outer",
                        {k: v for k, v in r.items() if k != "solves_per_s"})
    print(json.dumps(line), flush=True)
    return 0


def measure_c1(warmup, steps, m_reps=100):
    """c1: Wilson-clover 8^4, gauge eps 0.5, mass 0.1, csw 1.0: one Dslash (M)
    application and the plain eo2_ne CG to 1e-10 (maxiter 1000), FP64, with
    the oracle comparison.  Returns (summary dict, total solve ms)."""
    import torch

    import gpt_gb300 as g
    import oracle as o

    g.load()
    dims = [8, 8, 8, 8]
    grid = g.grid(dims, g.double)
    U = g.qcd.gauge.random_su3(grid, 0.5, 8)
    p = dict(mass=0.1, csw_r=1.0, csw_t=1.0, boundary_phases=[1.0, 1.0, 1.0, -1.0])
    op = g.qcd.fermion.wilson_clover(U, p)
    rng = np.random.default_rng(1)
    s = rng.standard_normal((grid.gsites, 4, 3)) + 1j * rng.standard_normal((grid.gsites, 4, 3))
    src = op.F_lattice()
    src[:] = s
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    cg = inv.cg({"eps": 1e-10, "maxiter": 1000})
    slv = inv.preconditioned(pc.eo2_ne(), cg)(op)
    out = op.F_lattice()
    for _ in range(max(1, warmup)):
        op.M(out, src)
        slv(src)
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    e[0].record(stream)
    for _ in range(m_reps):
        op.M(out, src)
    e[1].record(stream)
    for _ in range(steps):
        x = slv(src)
    e[2].record(stream)
    torch.cuda.synchronize()
    m_us = e[0].elapsed_time(e[1]) * 1000.0 / m_reps
    total_ms = e[1].elapsed_time(e[2])
    ref = o.wilson_clover(U.U, dims, **p)
    want = ref.apply("M", s)
    m_err = float(np.linalg.norm(out[:] - want) / np.linalg.norm(want))
    xr = x[:]
    tres = float(np.sqrt(o.norm2(s - ref.apply("M", xr)) / o.norm2(s)))
    return {"solves_per_s": steps / (total_ms / 1000.0), "ms_per_solve": total_ms / steps,
            "M_application_us": m_us, "M_vs_oracle_rel": m_err, "cg_iterations": cg.last.iterations,
            "true_residual_oracle": tres}, total_ms


def run_c1(args):
    r, total_ms = measure_c1(args.warmup, args.steps)
    cfg = {"workload": "wilson_clover 8^4 gauge eps 0.5 mass 0.1 csw 1.0 bc [1,1,1,-1], 1 gaussian source, "
                       "one M application + plain FP64 eo2_ne CG to 1e-10", "lattice": [8, 8, 8, 8],
           "l2_policy": "small case: resident in L2 (reported, not a roofline number)", "parallelism": "replicas"}
    line = _common_line(METRIC, r["solves_per_s"], "solves/s", args, 1, total_ms, cfg, "f64",
                        {k: v for k, v in r.items() if k != "solves_per_s"})
    print(json.dumps(line), flush=True)
    return 0


# published numbers of the reference's own Dslash benchmark (benchmarks/dslash.py,
# Mobius Dhop on 64.32.32.32, Ls 12, one node of 4 A100-SXM4-40GB:
# benchmarks/reference/juwels_booster/dslash_n1.txt:57-64, 67-74)
DHOP_PUBLISHED = {"single": {"gflops": 11325.46, "eff_gbs": 7824.86},
                  "double": {"gflops": 5749.77, "eff_gbs": 7945.14},
                  "hardware": "4x A100-SXM4-40GB (one JUWELS Booster node)"}


def dwf_dhop_benchmark(reps=None, dims=None, precisions=("single", "double_float", "double")):
    """The reference's headline benchmark (benchmarks/dslash.py) on one GPU:
    Mobius (mass 0.08, M5 1.8, b 1.5, c 0.5, Ls 12, periodic) Dhop on the
    full 5D field of a 64.32.32.32 lattice (or `dims`), N applications after
    5 warm-up ones, in each of `precisions` (single, double_float, double,
    half); flops = 1320 per 5D site and 'effective GB/s' = (8*2*4*3 +
    8*2*9/Ls + 2*4*3) reals per 5D site, the reference's models
    (dslash.py:54-61).  The algorithmic GB/s beside them counts each
    neighbour spinor once (L2 serves the eightfold reuse) and the links once
    per 4D site."""
    import torch

    import gpt_gb300 as g

    L = g.load()
    dims, Ls = dims or [64, 32, 32, 32], 12
    reps = reps or {"single": 1000, "double": 50, "double_float": 200}
    grid = g.grid(dims, g.double)
    U = g.qcd.gauge.random_su3_device(grid, 0.5, 777)
    params = dict(mass=0.08, M5=1.8, b=1.5, c=0.5, Ls=Ls, boundary_phases=[1.0, 1.0, 1.0, 1.0])
    V = grid.gsites
    sites = V * Ls
    stream = torch.cuda.current_stream()
    out = {"workload": "mobius Dhop, full 5D field, %s Ls 12 (benchmarks/dslash.py)" % ".".join(map(str, dims)),
           "published_reference": DHOP_PUBLISHED}
    for name, prec, sb, lb in (("single", g.single, 96, 48), ("double_float", g.double_float, 192, 144),
                               ("double", g.double, 192, 144), ("half", g.half, 52, 48)):
        if name not in precisions:
            continue
        op = g.qcd.fermion.mobius(U, params)
        op = op if prec is g.double else op.converted(prec)
        src, dst = op.F_lattice(), op.F_lattice()
        nat = torch.empty(V * Ls * 24, dtype=torch.float64, device="cuda")
        g._lib.check(L.gbf_random_spinor(V * Ls * 12, 99, nat.data_ptr(), g.core.stream_ptr()))
        g._lib.check(L.gbf_field_import(src.layout.op, nat.data_ptr(), src.ptr, 0, 1, g.core.stream_ptr()))
        del nat
        n = reps[name]
        for _ in range(5):
            op.Dhop.mat(dst, src)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            op.Dhop.mat(dst, src)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / n
        wbytes = {"single": 4, "half": 2}.get(name, 8)
        eff = (8 * 2 * 4 * 3 + 8 * 2 * 9 / Ls + 2 * 4 * 3) * wbytes * sites
        alg = (sb + sb + 8 * lb / Ls) * sites
        r = {"applications": n, "ms_per_application": ms, "gflops": 1320.0 * sites / (ms / 1000.0) / 1e9,
             "eff_gbs_reference_model": eff / (ms / 1000.0) / 1e9, "algorithmic_gbs": alg / (ms / 1000.0) / 1e9}
        pub = DHOP_PUBLISHED.get("double" if name == "double_float" else name)
        if pub:
            r["gflops_over_published_node"] = r["gflops"] / pub["gflops"]
        out[name] = r
        del op, src, dst
        torch.cuda.empty_cache()
    return out


def run_profile_dhop(args):
    """--profile-dhop: the Dhop benchmark's operator on a smaller lattice (by
    default 64.32.32.8, the benchmark's x3 slices with an eighth of its
    volume), one precision, 5 warm-up and 20 timed applications."""
    dims = [int(x) for x in args.dims.split(",")] if args.dims else [64, 32, 32, 8]
    r = dwf_dhop_benchmark({args.profile_precision: 20}, dims, (args.profile_precision,))
    print(json.dumps({"workload": r["workload"], args.profile_precision: r[args.profile_precision]}), flush=True)
    return 0


def run_dslash_bench(args):
    """--config dslash: the reference's own Dslash benchmark, one JSON line;
    value = FP32 GFlop/s (the published figure's precision)."""
    t0 = time.time()
    r = dwf_dhop_benchmark()
    line = {"metric": "DWF Dhop GFlop/s (benchmarks/dslash.py model, 1320 flop per 5D site)",
            "value": r["single"]["gflops"], "unit": "GFlop/s", "n_gpus": 1, "higher_is_better": True,
            "vs_baseline": r["single"]["gflops"] / DHOP_PUBLISHED["single"]["gflops"],
            "vs_baseline_note": "published figure is one node of 4 A100 GPUs; here one GB300",
            "dtype": "f32 (double and double-float alongside)", "data": "synthetic",
            "config": {"workload": r["workload"], "lattice": [64, 32, 32, 32], "Ls": 12},
            "seconds": time.time() - t0}
    line.update({k: v for k, v in r.items() if k not in ("workload",)})
    print(json.dumps(line), flush=True)
    return 0


def run_profile_next(args):
    """Profiling case of the kernels beyond the hot path, each launched a few
    times on inputs larger than L2: mode matrix (16 modes, Wilson 24^4 FP32
    half fields, 16 MB each), chiral shift and slice copy (Mobius 16^3x32
    Ls 12 FP32 full fields, 151 MB), multi-shift CG (Wilson-clover 24^4 FP64,
    4 shifts, 10 iterations), block CG (Mobius 12^3x24 Ls 12, 4 packed rhs,
    FP32, 5 iterations).  Prints the algorithmic bytes per launch of each."""
    import torch

    import gpt_gb300 as g
    from gpt_gb300 import core

    L = g.load()
    rng = np.random.default_rng(5)
    out = {}
    d24 = [24, 24, 24, 24]
    U24 = g.qcd.gauge.random_su3_device(g.grid(d24, g.double), 0.3, 21)
    wc = g.qcd.fermion.wilson_clover(U24, dict(mass=0.1, csw_r=1.0, csw_t=1.0, boundary_phases=[1, 1, 1, -1]))
    w32 = wc.converted(g.single)
    modes = [w32.F_lattice(core.odd) for _ in range(16)]
    for m_ in modes:
        m_.tensor.copy_(torch.randint(0, 255, m_.tensor.shape, dtype=torch.uint8, device="cuda") & 0x3F)
    src, dst = w32.F_lattice(core.odd), w32.F_lattice(core.odd)
    src.tensor.copy_(modes[1].tensor)
    mm = g.algorithms.modes.matrix(modes, modes, list(np.linspace(0.1, 1.0, 16)), lambda v: 1.0 / v)
    for _ in range(3):
        mm(dst, src)
    hb = w32.F_layout.half_bytes()
    out["mode_dot_kernel_bytes"] = 9 * hb
    out["mode_axpy_kernel_bytes"] = [9 * hb, 10 * hb]
    d5 = [16, 16, 16, 32]
    U5 = g.qcd.gauge.random_su3_device(g.grid(d5, g.double), 0.4, 22)
    qm = g.qcd.fermion.mobius(U5, dict(mass=0.01, M5=1.8, b=1.5, c=0.5, Ls=12, boundary_phases=[1, 1, 1, -1])).converted(g.single)
    qs = g.qcd.fermion.mobius(U5, dict(mass=0.01, M5=1.8, b=1.5, c=0.5, Ls=6, boundary_phases=[1, 1, 1, -1])).converted(g.single)
    a, b = qm.F_lattice(), qm.F_lattice()
    c = qs.F_lattice()
    a.tensor.copy_(torch.randint(0, 255, a.tensor.shape, dtype=torch.uint8, device="cuda") & 0x3F)
    for _ in range(3):
        g._lib.check(L.gbf_chiral_shift(a.layout.op, a.ptr, b.ptr, 1, 2, core.stream_ptr()))
        g._lib.check(L.gbf_copy_slices(c.layout.op, c.ptr, 0, a.layout.op, a.ptr, 3, 6, -1.0, 2, core.stream_ptr()))
    out["chiral_shift_kernel_bytes_per_half"] = 2 * a.layout.half_bytes()
    out["copy_slices_kernel_bytes_per_half"] = 2 * c.layout.half_bytes()
    Mpc = g.qcd.fermion.preconditioner.eo2_ne()(wc).Mpc
    F = wc.F_lattice()
    V = int(np.prod(d24))
    F[:] = rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3))
    bsrc = F.half(core.odd)
    ms = g.algorithms.inverter.multi_shift_cg({"eps": 1e-30, "maxiter": 10, "shifts": [0.01, 0.05, 0.2, 1.0]})
    ms(Mpc)(bsrc)
    out["multishift_kernel_bytes"] = (1 + 4 * 4) * wc.F_layout.half_bytes()
    d3 = [12, 12, 12, 24]
    U3 = g.qcd.gauge.random_su3_device(g.grid(d3, g.double), 0.4, 23)
    qb = g.qcd.fermion.mobius_operator(U3, dict(Ls=12, b=1.5, c=0.5, M5=1.8, mass_plus=0.01, mass_minus=0.01,
                                                boundary_phases=[1, 1, 1, -1], n_rhs=4), precision=g.single)
    sb = qb.F_lattice()
    nat = torch.empty(int(np.prod(d3)) * 12 * 24, dtype=torch.float64, device="cuda")
    for k in range(4):
        g._lib.check(L.gbf_random_spinor(int(np.prod(d3)) * 12 * 12, 60 + k, nat.data_ptr(), core.stream_ptr()))
        g._lib.check(L.gbf_field_import(sb.layout.op, nat.data_ptr(), sb.ptr, k, 1, core.stream_ptr()))
    xb = qb.F_lattice()
    qb._solve_eo2ne_block_cg(xb, sb, 1e-30, 5)
    hb5 = qb.F_layout.half_bytes()
    out["gram_kernel_bytes"] = 2 * hb5
    out["lincomb_kernel_bytes"] = 3 * hb5
    out["lincomb2_kernel_bytes"] = 6 * hb5
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "kernels beyond the hot path", **out}))
    return 0


def run_next_rows(args):
    """--config next: the measurements of next_rows_measurements() as one line."""
    t0 = time.time()
    out = next_rows_measurements()
    line = {"metric": "rows beyond the hot path: kernel GB/s, solver speed-ups, IO MB/s", "value": None,
            "unit": None, "n_gpus": 1, "data": "synthetic", "config": {"workload": "see each entry"},
            "block_cg": "measured by --config c3 --solver block_cg", "seconds": time.time() - t0}
    line.update(out)
    print(json.dumps(line), flush=True)
    return 0


def next_rows_measurements():
    """One measurement per row beyond the hot path, on synthetic inputs
    (gauge exp(i eps H), Gaussian sources), CUDA-event timing after warm-up.
    Algorithmic bytes count every field once per kernel (the hop: input
    spinor, 8 links, output, plus X and the site-local terms), as for the
    main roofline figure."""
    import tempfile

    import torch

    import gpt_gb300 as g
    from gpt_gb300 import core

    L = g.load()
    stream = torch.cuda.current_stream()
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)

    def timed(fn, n, warm=2):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    def gbs(nbytes, ms):
        return {"ms": ms, "algorithmic_gbs": nbytes / (ms / 1000.0) / 1e9, "frac_of_hbm_peak": nbytes / (ms / 1000.0) / 1e9 / peak}

    out = {}
    rng = np.random.default_rng(3)
    t_all = time.time()

    # ---- twisted-mass vs Wilson-clover M (32^4, FP32 and FP64) ----
    dims = [32, 32, 32, 32]
    U = g.qcd.gauge.random_su3_device(g.grid(dims, g.double), 0.3, 11)
    Vh = int(np.prod(dims)) // 2
    src4 = rng.standard_normal((2 * Vh, 4, 3)) + 1j * rng.standard_normal((2 * Vh, 4, 3))
    res = {}
    for prec, sb, lb in ((g.single, 96, 48), (g.double, 192, 144)):
        for kind in ("wilson_clover", "wilson_twisted_mass"):
            if kind == "wilson_clover":
                op = g.qcd.fermion.wilson_clover(U, dict(mass=0.05, csw_r=1.0, csw_t=1.0, boundary_phases=[1, 1, 1, -1]))
                local_b = 3 * sb  # clover: 288 / 576 B per site
            else:
                op = g.qcd.fermion.wilson_twisted_mass(U, dict(mass=0.05, mu=0.1, boundary_phases=[1, 1, 1, -1]))
                local_b = 0
            op = op if prec is g.double else op.converted(prec)
            x, y = op.F_lattice(), op.F_lattice()
            x[:] = src4
            ms = timed(lambda: op.M(y, x), 20)
            # M on both parities: out = Dhop(in) + Mooee in, per output site
            # in 8 neighbours once + 8 links + out + X (+ clover)
            nb = 2 * Vh * (sb + 8 * lb + sb + sb + local_b)
            res[f"{kind}_{prec.name}"] = gbs(nb, ms)
    out["twisted_mass_M_32^4"] = res

    # ---- zmobius vs mobius M (16^3x32, Ls 10, FP32) ----
    dims5 = [16, 16, 16, 32]
    U5 = g.qcd.gauge.random_su3_device(g.grid(dims5, g.double), 0.4, 12)
    omega = [0.17661651536320583 + 0.14907774771612217j, 0.23027432016909377 - 0.03530801572584271j,
             0.3368765581549033, 0.7305711010541054, 1.1686138337986505 + 0.3506492418109086j,
             1.1686138337986505 - 0.3506492418109086j, 0.994175013717952, 0.5029903152251229,
             0.23027432016909377 + 0.03530801572584271j, 0.17661651536320583 - 0.14907774771612217j]
    qm = g.qcd.fermion.mobius(U5, dict(mass=0.01, M5=1.8, b=1.5, c=0.5, Ls=10, boundary_phases=[1, 1, 1, -1]))
    qz = g.qcd.fermion.zmobius(U5, dict(mass=0.01, M5=1.8, b=1.0, c=0.0, omega=omega, boundary_phases=[1, 1, 1, -1]))
    res = {}
    for name, op in (("mobius", qm), ("zmobius", qz)):
        o32 = op.converted(g.single)
        x, y = o32.F_lattice(), o32.F_lattice()
        res[name + "_single_M_ms"] = timed(lambda: o32.M(y, x), 20)
    res["zmobius_over_mobius"] = res["zmobius_single_M_ms"] / res["mobius_single_M_ms"]
    out["zmobius_M_16^3x32_Ls10"] = res

    # ---- multi-shift CG (Wilson-clover 24^4, FP64, 8 shifts) vs 8 single-shift solves ----
    d24 = [24, 24, 24, 24]
    U24 = g.qcd.gauge.random_su3_device(g.grid(d24, g.double), 0.3, 13)
    w24 = g.qcd.fermion.wilson_clover(U24, dict(mass=0.1, csw_r=1.0, csw_t=1.0, boundary_phases=[1, 1, 1, -1]))
    Mpc = g.qcd.fermion.preconditioner.eo2_ne()(w24).Mpc
    b = w24.F_lattice(core.odd)
    F = w24.F_lattice()
    F[:] = rng.standard_normal((int(np.prod(d24)), 4, 3)) + 1j * rng.standard_normal((int(np.prod(d24)), 4, 3))
    b.tensor.copy_(F.half(core.odd).tensor)
    shifts = [1e-4, 3e-4, 1e-3, 3e-3, 1e-2, 3e-2, 0.1, 0.3]
    inv = g.algorithms.inverter
    ms_all = inv.multi_shift_cg({"eps": 1e-8, "maxiter": 5000, "shifts": shifts})
    msx = ms_all(Mpc)
    t_multi = timed(lambda: msx(b), 2, warm=1)
    it_multi = ms_all.last.iterations
    singles = [inv.multi_shift_cg({"eps": 1e-8, "maxiter": 5000, "shifts": [s]}) for s in shifts]
    sx = [m(Mpc) for m in singles]
    t_single = timed(lambda: [m(b) for m in sx], 1, warm=1)
    out["multi_shift_cg_24^4_fp64_8_shifts"] = {
        "ms_per_multishift_solve": t_multi, "iterations": it_multi, "ms_for_8_single_shift_solves": t_single,
        "iterations_single": [m.last.iterations for m in singles], "speedup": t_single / t_multi}

    # ---- deflation kernels: mode matrix with 32 modes on a 32^4 FP32 half field ----
    w32 = g.qcd.fermion.wilson_clover(U, dict(mass=0.05, csw_r=1.0, csw_t=1.0, boundary_phases=[1, 1, 1, -1])).converted(g.single)
    nev = 32
    modes = [w32.F_lattice(core.odd) for _ in range(nev)]
    for m_ in modes:
        m_.tensor.copy_(torch.randint(0, 255, m_.tensor.shape, dtype=torch.uint8, device="cuda") & 0x3F)
    src = w32.F_lattice(core.odd)
    src.tensor.copy_(modes[0].tensor)
    mm = g.algorithms.modes.matrix(modes, modes, list(np.linspace(0.1, 1.0, nev)), lambda v: 1.0 / v)
    dst = w32.F_lattice(core.odd)
    t_modes = timed(lambda: mm(dst, src), 5)
    hb = w32.F_layout.half_bytes()
    blocks = (nev + 7) // 8
    nbytes = (nev + blocks) * hb + (nev + blocks + (blocks - 1)) * hb
    out["deflation_mode_matrix_32^4_fp32_32_modes"] = gbs(nbytes, t_modes)

    # ---- MADWF moves and a MADWF solve (16^3x32: Mobius Ls 12 outer, zmobius Ls 10 inner) ----
    qm12 = g.qcd.fermion.mobius(U5, dict(mass=0.01, M5=1.8, b=1.5, c=0.5, Ls=12, boundary_phases=[1, 1, 1, -1]))
    q32 = qm12.converted(g.single)
    a, c_ = q32.F_lattice(), q32.F_lattice()
    t_shift = timed(lambda: L.gbf_chiral_shift(a.layout.op, a.ptr, c_.ptr, 1, 2, core.stream_ptr()), 20)
    out["madwf_chiral_shift_16^3x32_Ls12_fp32"] = gbs(2 * a.tensor.numel(), t_shift)
    pc = g.qcd.fermion.preconditioner
    inner_cg = inv.preconditioned(pc.eo2_ne(), inv.cg({"eps": 1e-5, "maxiter": 4000}))
    qz32 = qz.converted(g.single)
    madwf = inv.defect_correcting(inv.mixed_precision(pc.mixed_dwf(inner_cg, inner_cg, qz32), g.single, g.double),
                                  eps=1e-8, maxiter=30)
    plain = inv.defect_correcting(inv.mixed_precision(inner_cg, g.single, g.double), eps=1e-8, maxiter=30)
    S = qm12.U_lattice()
    S[:] = rng.standard_normal((int(np.prod(dims5)), 4, 3)) + 1j * rng.standard_normal((int(np.prod(dims5)), 4, 3))
    res = {}
    for name, slv in (("madwf_zmobius_Ls10_inner", madwf), ("mixed_precision_cg", plain)):
        prop = qm12.propagator(slv)
        t0 = time.time()
        x4 = prop(S)
        torch.cuda.synchronize()
        res[name] = {"s_per_solve": time.time() - t0, "outer_corrections": len(slv.history)}
    out["madwf_solve_16^3x32_mobius_Ls12_to_1e-8"] = res

    # ---- gauge-field IO (32^4 FP64, 604 MB) ----
    H = U.host()
    nbytes = H.nbytes
    res = {}
    with tempfile.TemporaryDirectory() as d:
        for name, fmt in (("nersc", g.format.nersc()), ("ildg", g.format.ildg()), ("lime", g.format.lime())):
            fn = os.path.join(d, name)
            t0 = time.time()
            g.save(fn, U, fmt)
            t1 = time.time()
            V = g.load(fn)
            t2 = time.time()
            assert np.array_equal(V.host(), H)
            res[name] = {"save_MBps": nbytes / (t1 - t0) / 1e6, "load_MBps": nbytes / (t2 - t1) / 1e6}
            os.remove(fn)
    out["gauge_io_32^4_fp64"] = res

    out["seconds"] = time.time() - t_all
    return out


def measure_c5(n_requests, rate=20.0):
    """c5: Poisson stream at `rate` req/s of Wilson-clover propagator
    requests, L in {8,16,24,32}, gauge eps U[0.2,0.5], mass U[0.01,0.2], 1-12
    sources, true residual 1e-10, mixed method with continuous batching.
    Beside it: (1) the same stream served strictly one request at a time with
    the plain FP64 CG (the serial baseline), and (2) a sustainable-rate point:
    a stream of the same mix offered at 3/4 of the request rate the server
    reached at `rate`, where the served rate follows the offered one and the
    latencies do not grow with the stream's length.  Returns (summary dict,
    wall ms of the main stream, config dict)."""
    import torch

    import gpt_gb300 as g
    from gpt_gb300 import serving

    g.load()
    reqs = serving.poisson_stream(n_requests, rate, seed=2026)
    free, total = torch.cuda.mem_get_info()
    budget = int(0.8 * free)
    ex = serving.gpu_executor()
    # warm-up: one small request of every size (library, graphs, allocator)
    serving.Server(ex, budget, realtime=False).run([serving.Request(-1 - i, L, 0.3, 5, 0.1, 1, 6)
                                                     for i, L in enumerate([8, 16, 24, 32])])
    L = g._lib.load()
    n0 = L.gbf_launch_count()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    res, wall = serving.Server(ex, budget, method="mixed").run(reqs)
    clk = clocks.stop()
    n1 = L.gbf_launch_count()
    s = serving.summarize(res, wall)

    def above(rs):
        return [(r.rid, r.L, r.n_src, max(r.true_residual)) for r in rs if r.true_residual and max(r.true_residual) > 1e-10]

    def errors(rs):
        return [(r.rid, r.L, r.n_src, r.error[:200]) for r in rs if not r.ok][:4]

    # serial baseline: the same stream, one request at a time (max_total 1),
    # plain FP64 eo2_ne CG, drained in arrival order
    serial, swall = serving.Server(ex, budget, method="plain", realtime=False, max_total=1).run(reqs)
    ss = serving.summarize(serial, swall)
    # sustainable point: the same mix offered at 3/4 of the saturated request rate
    srate = 0.75 * s["requests_per_s"]
    sreqs = serving.poisson_stream(n_requests, srate, seed=2027)
    sres, sw = serving.Server(ex, budget, method="mixed").run(sreqs)
    su = serving.summarize(sres, sw)
    offered = n_requests / sreqs[-1].arrival
    cfg = {"workload": f"serving: {n_requests} Poisson requests at {rate:g}/s, wilson_clover L^4 L in {{8,16,24,32}}, "
                       "gauge eps U[0.2,0.5], mass U[0.01,0.2], 1-12 gaussian sources, true residual 1e-10; "
                       "mixed method with HBM-footprint admission and batching by lattice size",
           "hbm_budget_bytes": budget, "l2_policy": "per-request working sets; no flush", "parallelism": "replicas"}
    r = {"solves_per_s": s["solves_per_s"], "requests_per_s": s["requests_per_s"],
         "offered_requests_per_s": n_requests / reqs[-1].arrival, "p50_ms": s["p50_ms"], "p99_ms": s["p99_ms"],
         "failed": s["failed"], "errors": errors(res), "max_true_residual": s["max_true_residual"],
         "mixed_above_tol": above(res),
         "gpu_launches": int(n1 - n0), "clocks": clk,
         "serial_plain_fp64": {"note": "the same stream served one request at a time (no overlap), plain FP64 CG",
                               "solves_per_s": ss["solves_per_s"], "wall_s": swall, "p50_ms": ss["p50_ms"],
                               "p99_ms": ss["p99_ms"], "failed": ss["failed"], "errors": errors(serial),
                               "max_true_residual": ss["max_true_residual"],
                               "above_tol": above(serial)},
         "speedup_vs_serial_plain": s["solves_per_s"] / ss["solves_per_s"] if ss["solves_per_s"] else None,
         "sustainable_point": {"offered_requests_per_s": offered, "served_requests_per_s": su["requests_per_s"],
                               "solves_per_s": su["solves_per_s"], "p50_ms": su["p50_ms"], "p99_ms": su["p99_ms"],
                               "failed": su["failed"], "errors": errors(sres),
                               "max_true_residual": su["max_true_residual"]}}
    return r, 1000.0 * wall, cfg


def other_config_measurements():
    """The configurations beside the headline one, compact, for the default
    line: c1 (8^4 Wilson-clover), c3 (Mobius 16^3x32 Ls 12, 12 point
    sources, FP32 and FP16 inner), c4 (Mobius 32^3x64 Ls 16: one packed group
    of 2 of its 12 Gaussian sources) and c5 (a 40-request serving stream).
    Every solve's FP64 oracle residual is reported (c3, c4: every 5D system
    of the timed step; c1: the solution)."""
    import torch

    out = {}

    def clean():
        gc.collect()
        torch.cuda.empty_cache()

    def keep(r, drop=("clocks", "rhs_group_tuning", "device_memory_total_gb", "gpu_launches")):
        return {k: v for k, v in r.items() if k not in drop}

    t0 = time.time()
    try:
        r, _ = measure_c1(3, 20)
        out["c1"] = {"workload": "wilson_clover 8^4, one M + plain FP64 eo2_ne CG to 1e-10", **r}
    except Exception as e:
        out["c1"] = {"error": f"{type(e).__name__}: {e}"}
    clean()
    c3 = {"workload": "mobius 16^3x32 Ls 12, 12 point sources packed, defect correction to true residual 1e-8; "
                      "one warm-up and one timed 12-source propagator per inner precision"}
    for inner in ("single", "half"):
        try:
            r, _, _ = measure_mobius("c3", 1, 1, inner=inner)
            c3[f"{inner}_inner"] = keep(r)
        except Exception as e:
            c3[f"{inner}_inner"] = {"error": f"{type(e).__name__}: {e}"}
        clean()
    out["c3"] = c3
    try:
        r, _, _ = measure_mobius("c4", 0, 1, inner="single", rhs_group=2, max_groups=1)
        out["c4"] = {"workload": "mobius 32^3x64 Ls 16 mass 0.005, one packed group of 2 of the 12 gaussian sources, "
                                 "FP32 inner / FP64 outer to true residual 1e-10 (first solve: includes graph capture)",
                     "seconds_per_source": r["ms_per_solve"] / 1000.0, **keep(r)}
    except Exception as e:
        out["c4"] = {"error": f"{type(e).__name__}: {e}"}
    clean()
    try:
        r, _, _ = measure_c5(40)
        out["c5"] = {"workload": "serving: 40 Poisson requests at 20/s, wilson_clover L in {8,16,24,32}^4, 1-12 "
                                 "sources each, to true residual 1e-10", **keep(r)}
    except Exception as e:
        out["c5"] = {"error": f"{type(e).__name__}: {e}"}
    clean()
    out["configs_seconds"] = time.time() - t0
    return out


def run_c5(args):
    r, wall_ms, cfg = measure_c5(args.requests)
    line = _common_line(METRIC, r["solves_per_s"], "solves/s", args, 1, wall_ms, cfg, "f32 inner / f64 outer",
                        {k: v for k, v in r.items() if k != "solves_per_s"})
    print(json.dumps(line), flush=True)
    return 0


def run_profile_case(args, dims):
    """A small-footprint run of the inner FP32 solve (about 1.5 GB on the
    device at 32^4) for ncu captures of the hopping kernel."""
    import torch

    import gpt_gb300 as g

    g.load()
    grid = g.grid(dims, g.double)
    U = g.qcd.gauge.random_su3(grid, CFG["gauge_eps"], CFG["gauge_seed"])
    params = dict(mass=CFG["mass"], csw_r=CFG["csw"], csw_t=CFG["csw"], boundary_phases=CFG["phases"])
    prec = {"single": g.single, "double": g.double, "double_float": g.double_float, "half": g.half}[args.profile_precision]
    op = g.qcd.fermion.wilson_clover_operator(U, params, precision=prec)
    V = grid.gsites
    rng = np.random.default_rng(CFG["src_seed"])
    src = op.F_lattice()
    src[:] = (rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3))) * 1e-3
    x = op.F_lattice()
    for _ in range(args.warmup):
        op._solve_eo2ne_cg(x, src, 1e-30, 12)
    torch.cuda.synchronize()
    r = op._solve_eo2ne_cg(x, src, 1e-30, 12)
    torch.cuda.synchronize()
    # the same solve once more with per-kernel-class timing (events around
    # the launches: hop, site-local, vector kernels)
    rp = op._solve_eo2ne_cg(x, src, 1e-30, 12, 0, 1)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": f"wilson_clover {args.profile_precision} eo2_ne CG, 12 iterations", "lattice": dims,
                      "iterations": r.iterations, "link_bytes": op.link_bytes(),
                      "kernel_ms": list(rp.kernel_ms), "kernel_launches": list(rp.kernel_launches)}))
    return 0


def workload_config(dims):
    return {
        "workload": f"wilson_clover {'x'.join(map(str, dims))} gauge exp(i*{CFG['gauge_eps']}*H) mass {CFG['mass']} "
                    f"csw {CFG['csw']} bc [1,1,1,-1], 1 gaussian source, eo2_ne CG: mixed FP32-inner (tol "
                    f"{CFG['inner_tol']}) + FP64 defect correction to true residual {CFG['tol']}",
        "lattice": dims,
        "precision": "FP32 inner / FP64 outer (value), FP64 plain alongside",
        "l2_policy": "inputs larger than L2 (gauge 604 MB, clover 1.2 GB, FP64 source 201 MB); no flush",
        "parallelism": "replicas (one independent solve stream per GPU)",
    }


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def run_reference(args, dims):
    """--impl reference: the CPU restatement of the same mixed solve (the
    reference's Grid CPU operator cannot be built here) on all host cores;
    every step is one full solve of the workload, timed."""
    import oracle as o
    from gpt_gb300.qcd import gauge as G
    import gpt_gb300.core as core

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    grid = core.grid.__new__(core.grid)
    grid.fdimensions, grid.gsites, grid.precision = dims, int(np.prod(dims)), None
    U = G.random_su3(grid, CFG["gauge_eps"], CFG["gauge_seed"]).U
    rng = np.random.default_rng(CFG["src_seed"])
    V = int(np.prod(dims))
    src = rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3))
    op = o.wilson_clover(U, dims, mass=CFG["mass"], csw_r=CFG["csw"], csw_t=CFG["csw"],
                         boundary_phases=CFG["phases"], with_single=True)

    def solve():
        return op.defect_correcting(src, CFG["tol"], 50, CFG["inner_tol"], 100000)

    for _ in range(args.warmup):
        solve()
    secs = []
    tstart = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        x, inner_it, n_outer, tres = solve()
        secs.append(time.perf_counter() - t0)
    wall = time.perf_counter() - tstart
    value = args.steps / wall
    cores = o.num_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * wall / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 outer",
        "data": "synthetic", "config": workload_config(dims),
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": f"every step one full mixed solve on the host cores (oracle: single-precision "
                                   f"eo2_ne CG inner, FP64 defect correction): {inner_it} inner iterations, "
                                   f"{n_outer} outer corrections, true residual {tres:.2e}, median "
                                   f"{statistics.median(secs):.2f} s per solve"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gbf(args, dims):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import gpt_gb300 as g

    L = g.load()
    grid = g.grid(dims, g.double)
    U = g.qcd.gauge.random_su3(grid, CFG["gauge_eps"], CFG["gauge_seed"] + rank)
    params = dict(mass=CFG["mass"], csw_r=CFG["csw"], csw_t=CFG["csw"], boundary_phases=CFG["phases"])
    op = g.qcd.fermion.wilson_clover(U, params)
    inv = g.algorithms.inverter
    pc = g.qcd.fermion.preconditioner
    cg_loop = {"iterations_per_graph": max(-1, args.cg_graph), "profile": args.cg_graph < -1}
    inner_cg = inv.cg({"eps": CFG["inner_tol"], "maxiter": 20000, **cg_loop})
    dc = inv.defect_correcting(inv.mixed_precision(inv.preconditioned(pc.eo2_ne(), inner_cg), g.single, g.double),
                               eps=CFG["tol"], maxiter=100)
    solver = dc(op)
    inner_op = dc.inner_inverter.inner_op  # the FP32 operator built by mixed_precision
    # the plain CG's eps bounds the eo2_ne normal residual; tol / 3 brings the
    # true residual of M x = b below tol (eps = tol leaves it at 1.5 tol)
    plain_cg = inv.cg({"eps": CFG["tol"] / 3, "maxiter": 40000, **cg_loop})
    plain = inv.preconditioned(pc.eo2_ne(), plain_cg)(op)

    V = grid.gsites
    rng = np.random.default_rng(CFG["src_seed"] + rank)
    src_np = rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3))
    src = op.F_lattice()
    src[:] = src_np
    stream = torch.cuda.current_stream()

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- warm-up ----
    for _ in range(args.warmup):
        x = solver(src)

    # ---- timed region: K mixed solves, source resident in HBM ----
    clocks = Clocks(local if "CUDA_VISIBLE_DEVICES" not in os.environ else local)
    clocks.start()
    barrier()
    n0 = L.gbf_launch_count()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    ev[0].record(stream)
    torch.cuda.nvtx.range_push("timed")  # ncu --nvtx --nvtx-include "timed/" captures this region only
    for k in range(args.steps):
        x = solver(src)
        ev[k + 1].record(stream)
    torch.cuda.nvtx.range_pop()
    barrier()
    n1 = L.gbf_launch_count()
    clk = clocks.stop()
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    total_ms = max_over_ranks(ev[0].elapsed_time(ev[args.steps]), dist, "cuda")
    value = whole_job_rate(world, args.steps, total_ms)

    # true residual of the last solve, FP64 on the device
    r = op.F_lattice()
    op.M(r, x)
    g.axpby(r, -1.0, r, 1.0, src)
    true_res = math.sqrt(g.norm2(r) / g.norm2(src))
    outer_iters = len(dc.history) - 1

    # inner CG iterations of one mixed solve (running total kept by the cg object)
    before = inner_cg.total_iterations
    x = solver(src)
    inner_iters_per_solve = inner_cg.total_iterations - before
    ns = g.norm2(src)

    # ---- e2e through the public API from pinned host memory ----
    h_src = torch.from_numpy(src_np.view(np.float64).reshape(-1)).pin_memory()
    h_dst = torch.empty(V * 24, dtype=torch.float64).pin_memory()
    d_nat = torch.empty(V * 24, dtype=torch.float64, device="cuda")
    e2e_steps = args.steps
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        d_nat.copy_(h_src, non_blocking=True)
        lat = op.F_lattice()
        g._lib.check(L.gbf_field_import(lat.layout.op, d_nat.data_ptr(), lat.ptr, 0, 0, g.core.stream_ptr()))
        xo = solver(lat)
        g._lib.check(L.gbf_field_export(xo.layout.op, xo.ptr, d_nat.data_ptr(), 0, 0, g.core.stream_ptr()))
        h_dst.copy_(d_nat, non_blocking=True)
    e1.record(stream)
    barrier()
    e2e_value = whole_job_rate(world, e2e_steps, max_over_ranks(e0.elapsed_time(e1), dist, "cuda"))

    # ---- plain FP64 eo2_ne CG ----
    xp = plain(src)  # warm-up (also builds the graph)
    plain_it = plain_cg.last.iterations
    barrier()
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for _ in range(args.plain_steps):
        xp = plain(src)
    p1.record(stream)
    barrier()
    plain_ms = p0.elapsed_time(p1) / args.plain_steps
    op.M(r, xp)
    g.axpby(r, -1.0, r, 1.0, src)
    plain_true = math.sqrt(g.norm2(r) / g.norm2(src))

    # ---- operator set-up: a Wilson-clover operator from a gauge field in HBM
    # (links packed, clover term built and inverted on the device) ----
    import torch as _t
    Ud = g.qcd.gauge.gauge_field(grid, _t.from_numpy(U.U.view(np.float64).reshape(-1)).to("cuda"))
    barrier()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    op_setup = g.qcd.fermion.wilson_clover(Ud, params)
    s1.record(stream)
    barrier()
    setup_ms = s0.elapsed_time(s1)
    del op_setup, Ud

    # ---- dominant kernel: FP32 hopping kernel inside the inner CG, timed with
    # CUDA events around every launch (profile-mode solve on the same stream) ----
    cs = inner_op.F_lattice()
    g.convert(cs, src, 1.0 / math.sqrt(ns))
    xd = inner_op.F_lattice()
    res32 = inner_op._solve_eo2ne_cg(xd, cs, CFG["inner_tol"], 400, 0, 1)
    d_ms = res32.kernel_ms[0] / max(1, res32.kernel_launches[0])
    Vh = V // 2
    link_b = inner_op.link_bytes()
    spin_b, clov_b = 96, 288
    # algorithmic bytes per output site, the four launches of one iteration:
    #   z = G Dhop t, w = p - Dhop z, u = G Dhop^+ w, mmp = w - G Dhop^+ u (+<p,mmp>)
    per_site = [spin_b + 8 * link_b + clov_b + spin_b,
                spin_b + 8 * link_b + spin_b + spin_b,
                spin_b + 8 * link_b + clov_b + spin_b,
                spin_b + 8 * link_b + clov_b + spin_b + spin_b + spin_b]
    bytes_per_launch = statistics.mean(per_site) * Vh
    achieved = bytes_per_launch / (d_ms / 1000.0) / 1e9
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    traffic = None
    tf = os.path.join(ROOT, "profiles", "dslash_fp32_traffic.json")
    if os.path.exists(tf):
        t = json.load(open(tf))
        traffic = t["dram_bytes_per_site"] * Vh

    # FP64 hopping kernel (plain method), same profile mode
    res64 = op._solve_eo2ne_cg(op.F_lattice(), src, CFG["tol"], 50, 0, 1)
    d64_ms = res64.kernel_ms[0] / max(1, res64.kernel_launches[0])
    per_site64 = statistics.mean([192 + 8 * 144 + 576 + 192, 192 + 8 * 144 + 192 + 192,
                                  192 + 8 * 144 + 576 + 192, 192 + 8 * 144 + 576 + 3 * 192])
    fp64_gbs = per_site64 * Vh / (d64_ms / 1000.0) / 1e9

    # ---- double-float (FP64-class on the FP32 pipe): plain CG, its hopping
    # kernel, and the mixed solve with a double-float outer loop ----
    op_dd = op.converted(g.double_float)
    src_dd = op_dd.F_lattice()
    src_dd[:] = src_np
    dd_cg = inv.cg({"eps": CFG["tol"] / 3, "maxiter": 40000})
    plain_dd = inv.preconditioned(pc.eo2_ne(), dd_cg)(op_dd)
    xq = plain_dd(src_dd)
    dd_it = dd_cg.last.iterations
    barrier()
    p0.record(stream)
    for _ in range(args.plain_steps):
        xq = plain_dd(src_dd)
    p1.record(stream)
    barrier()
    plain_dd_ms = p0.elapsed_time(p1) / args.plain_steps
    xf = op.F_lattice()
    g.convert(xf, xq)
    op.M(r, xf)
    g.axpby(r, -1.0, r, 1.0, src)
    plain_dd_true = math.sqrt(g.norm2(r) / g.norm2(src))
    resdd = op_dd._solve_eo2ne_cg(op_dd.F_lattice(), src_dd, CFG["tol"], 50, 0, 1)
    ddd_ms = resdd.kernel_ms[0] / max(1, resdd.kernel_launches[0])
    dd_gbs = per_site64 * Vh / (ddd_ms / 1000.0) / 1e9
    inner_dd = inv.cg({"eps": CFG["inner_tol"], "maxiter": 20000})
    dc_dd = inv.defect_correcting(inv.mixed_precision(inv.preconditioned(pc.eo2_ne(), inner_dd), g.single,
                                                      g.double_float), eps=CFG["tol"], maxiter=100)
    solver_dd = dc_dd(op_dd)
    xm = solver_dd(src_dd)
    barrier()
    p0.record(stream)
    for _ in range(args.steps):
        xm = solver_dd(src_dd)
    p1.record(stream)
    barrier()
    mixed_dd_ms = p0.elapsed_time(p1) / args.steps
    g.convert(xf, xm)
    op.M(r, xf)
    g.axpby(r, -1.0, r, 1.0, src)
    mixed_dd_true = math.sqrt(g.norm2(r) / g.norm2(src))
    del op_dd, src_dd, plain_dd, solver_dd, xq, xm

    if rank != 0:
        if dist is not None:
            dist.barrier()
        return 0

    # ---- CPU baseline (oracle port), rank 0 at N = 1 only ----
    cpu = None
    oracle_res = {}
    if world == 1 and not args.no_cpu_baseline:
        import oracle as o

        op_o = o.wilson_clover(U.U, dims, mass=CFG["mass"], csw_r=CFG["csw"], csw_t=CFG["csw"],
                               boundary_phases=CFG["phases"], with_single=True)
        # FP64 oracle residual of the mixed and the plain solutions
        for name, sol in (("mixed", x), ("plain", xp)):
            xs = sol[:]
            rr = src_np - op_o.apply("M", xs)
            oracle_res[name] = math.sqrt(o.norm2(rr) / o.norm2(src_np))
        # one full mixed solve of the same source on the host cores, timed
        t0 = time.perf_counter()
        _, c_inner, c_outer, c_res = op_o.defect_correcting(src_np, CFG["tol"], 50, CFG["inner_tol"], 100000)
        sec = time.perf_counter() - t0
        cpu = {"value": 1.0 / sec, "unit": "solves/s", "cores": o.num_threads(), "kind": "port",
               "sample": f"one full mixed solve of this workload (oracle: single-precision eo2_ne CG inner, FP64 "
                         f"defect correction) on the host cores: {c_inner} inner iterations, {c_outer} outer "
                         f"corrections, {sec:.1f} s, true residual {c_res:.2e}"}
        del op_o

    # ---- the reference's own Dslash benchmark (benchmarks/dslash.py), after the timed region ----
    dhop = nxt = None
    if world == 1 and not args.no_dhop_benchmark:
        try:
            dhop = dwf_dhop_benchmark()
        except Exception as e:  # reported, not fatal for the headline line
            dhop = {"error": f"{type(e).__name__}: {e}"}
    if world == 1 and not args.no_next_rows:
        try:
            nxt = next_rows_measurements()
        except Exception as e:
            nxt = {"error": f"{type(e).__name__}: {e}"}

    # ---- the other configurations, compact, after the timed region ----
    configs = {}
    if world == 1 and not args.no_configs:
        configs = other_config_measurements()

    p = sorted(step_ms)
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "solves/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 inner / f64 outer",
        "data": "synthetic",
        "config": workload_config(dims),
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": V * 12 * 16,
                "d2h_bytes_per_step": V * 12 * 16, "steps": e2e_steps},
        "gpu_launches": int(n1 - n0),
        "clocks": clk,
        "roofline": {"bound": "hbm", "kernel": "dslash_kernel<FP32 spinor, 12-real links, clover epilogue>",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
                     "algorithmic_bytes_per_launch": bytes_per_launch, "avg_launch_ms": d_ms},
        "cpu_baseline": cpu,
        # ---- detail first; the figures to read last (end of the line) ----
        "reference_dslash_benchmark": dhop,
        "rows_beyond_the_hot_path": nxt,
        "cg_loop": ("host-checked CUDA graphs of 16 iterations" if args.cg_graph == 0 else
                    f"host-checked CUDA graphs of {args.cg_graph} iterations" if args.cg_graph > 0 else
                    "device: one CUDA graph with a conditional while node" if args.cg_graph == -1 else
                    "no graphs: host launches with CUDA events (diagnostic)"),
        "p50_ms": p[len(p) // 2],
        "p99_ms": p[min(len(p) - 1, int(math.ceil(0.99 * len(p))) - 1)],
        **configs,
        "double_float": {
            "note": "FP64-class precision on the FP32 pipe: every real is h + l of two FP32 words (48-bit "
                    "significand); M agrees with the FP64 operator to about 7e-15 relative",
            "dslash": {"algorithmic_gbs": dd_gbs, "avg_launch_ms": ddd_ms, "frac_of_hbm_peak": dd_gbs / peak},
            "plain_cg": {"solves_per_s": world * 1000.0 / plain_dd_ms, "ms_per_solve": plain_dd_ms,
                         "cg_iterations": dd_it, "true_residual_fp64": plain_dd_true},
            "mixed_single_inner": {"solves_per_s": world * 1000.0 / mixed_dd_ms, "ms_per_solve": mixed_dd_ms,
                                   "true_residual_fp64": mixed_dd_true},
        },
        "operator_setup_ms": {"wilson_clover_32^4_fp64": setup_ms,
                              "note": "gauge field in HBM -> packed links, clover term and its inverse (FP64 + FP32)"},
        "dslash_fp32": {"hbm_gbs": achieved, "avg_launch_ms": d_ms, "frac_of_hbm_peak": achieved / peak},
        "dslash_fp64": {"algorithmic_gbs": fp64_gbs, "avg_launch_ms": d64_ms, "frac_of_hbm_peak": fp64_gbs / peak,
                        "gflops_model_1320_per_site": 1320 * Vh / (d64_ms / 1000.0) / 1e9,
                        "bound": "FP64 pipe (about 1.0 TFLOP/s measured on GB300)"},
        "mixed": {"solves_per_s": value, "true_residual": true_res, "true_residual_oracle": oracle_res.get("mixed"),
                  "outer_corrections": outer_iters, "inner_cg_iterations": inner_iters_per_solve},
        "plain_fp64": {"solves_per_s": world * 1000.0 / plain_ms, "ms_per_solve": plain_ms, "cg_iterations": plain_it,
                       "true_residual": plain_true, "true_residual_oracle": oracle_res.get("plain")},
        "mixed_over_plain": (value / world) / (1000.0 / plain_ms),
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    dims = [int(d) for d in args.dims.split(",")] if args.dims else CFG["dims"]
    if args.profile_dslash:
        return run_profile_case(args, dims)
    if args.profile_mobius:
        return run_profile_mobius(args)
    if args.profile_dhop:
        return run_profile_dhop(args)
    if args.profile_next:
        return run_profile_next(args)
    if args.impl != "reference" and args.config == "c1":
        return run_c1(args)
    if args.impl != "reference" and args.config in ("c3", "c4"):
        return run_mobius_config(args, args.config)
    if args.impl != "reference" and args.config == "c5":
        return run_c5(args)
    if args.impl != "reference" and args.config == "next":
        return run_next_rows(args)
    if args.impl != "reference" and args.config == "dslash":
        return run_dslash_bench(args)
    if args.impl == "reference":
        return run_reference(args, dims)
    return run_gbf(args, dims)


if __name__ == "__main__":
    sys.exit(main())
