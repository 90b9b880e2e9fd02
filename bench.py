"""Benchmark: converged cells/sec of the PRISM-3D steady state on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload slab128] [--plain full|estimate|auto]

Workload (default): the 128^3 Orion-Bar-like slab -- n_H rising as a tanh
ramp from 1e3 to 1e5 cm^-3 along x over ~0.05 pc times a seeded log-normal
perturbation (sigma_ln 0.8), G0 = 2.6e4 on the -x face, 48 rays (nside 2),
zeta = 2e-16, 0.005 pc cells, T_init = 100 K.  Synthetic, seeded inputs
(prism3d_gb300/fields.py); no dataset is involved.

One step = one full solve from the initial state to outer convergence
(p3d_steady_reset + p3d_steady_run, mixed precision): the ray march, the
per-cell constants and initial abundances, then outer iterations until at
most max(8, 1e-5 n) cells change by more than 1e-8.
  value      n_cells / mean step time, device-resident inputs, CUDA events
             on the library stream; the per-step state (~35 doubles per cell,
             0.6 GB at 128^3) exceeds the 126 MB L2, so no flush is needed.
  e2e        the same through the C ABI from host buffers: p3d_steady_create
             (density and tables host->device) + reset + run + p3d_steady_get
             of the 8 state fields, wall clock.
  plain      the plain FP64 path (same algorithm, FP64 everywhere, no warm
             starts or compaction, host-checked every iteration): its own
             full solve and the per-species difference of the mixed state
             from it (--plain full; the default up to 2^21 cells, ~100 s at
             128^3), or the per-iteration time over a bounded sample of
             iterations (--plain estimate; the default above 2^21 cells).
  cpu_baseline / --impl reference: the CPU oracle (C restatement of the
             reference's kernels with OpenMP + NumPy ray march) timing one
             reference outer iteration (solver_3d.py:262-376 with the Rust
             core's explicit-Euler chemistry) on the full grid with all host
             cores, scaled by the iteration count of the GPU solve.
With --gpus N > 1 (torchrun), each rank solves its own independent replica
(the path has no exchange step on one box): value is the sum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "converged cells/sec at 128^3 (batched mixed vs plain FP64 GPU, <=1e-6 rel err)"


def max_over_ranks(value, ws, device="cpu"):
    """Largest value over the ranks of the process group (the step time of the
    slowest replica); the value itself with one rank."""
    if ws <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampler for the timed region (SM clock, throttle reasons)."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def __enter__(self):
        def loop():
            while not self._stop.is_set():
                try:
                    out = subprocess.run(
                        ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                         "--format=csv,noheader,nounits"], capture_output=True, text=True,
                        timeout=5).stdout.strip()
                    if out:
                        self.rows.append([v.strip() for v in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=loop, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)

    def summary(self):
        import statistics
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if len(r) > 3 + k and r[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def run_gb300(args, ws, rank, local):
    import numpy as np
    import torch

    from prism3d_gb300 import fields
    from prism3d_gb300 import _lib as L
    from prism3d_gb300.solver import PDRSolverGPU

    torch.cuda.set_device(local)
    dens, g0, nside, zeta, cell = fields.workload(args.workload, seed=1 + rank)
    n = dens.size
    box = cell * dens.shape[0]
    s = PDRSolverGPU(dens, box, G0_external=g0, zeta_CR_0=zeta, nside_rt=nside, T_init=100.0)
    n_allow = max(8, int(1e-5 * n))

    def solve(mixed=True, max_it=4000):
        s.reset()
        return s.run(max_iterations=max_it, convergence_tol=args.tol, mixed=mixed, n_allow=n_allow,
                     w_chem=args.w_chem)

    tuned = s.autotune()  # launch shape of the per-cell kernels (untimed)
    for _ in range(args.warmup):
        solve()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    times, iters, oks, launches = [], [], [], []
    with Clocks(local) as clk:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            ok = solve()
            times.append(s.elapsed_ms() * 1e-3)
            iters.append(s.iterations)
            oks.append(bool(ok))
            launches.append(s.launch_count())
    if ws > 1:
        torch.distributed.barrier()
    t_step = max_over_ranks(float(np.mean(times)), ws, "cuda")
    value = n * ws / t_step
    hist = s.convergence_history()
    # e2e through the C ABI from host buffers: a new solver on the host
    # density (device state allocated, inputs and tables uploaded, ray march),
    # the solve, the state read back; the one-time grain tables and the
    # launch shape autotune() chose are reused, as a caller solving grid
    # after grid would
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s2 = PDRSolverGPU(dens, box, G0_external=g0, zeta_CR_0=zeta, nside_rt=nside, T_init=100.0,
                      tables=s.tables)
    s2.set_launch(tuned[0], tuned[1])
    s2.run(max_iterations=4000, convergence_tol=args.tol, mixed=True, n_allow=n_allow,
           w_chem=args.w_chem)
    outs = [s2.get(k) for k in STATE_KEYS]
    t_e2e = time.perf_counter() - t0
    chg_mixed = s2.get("change")
    refine = None
    if args.network_cells > 0:
        # refinement pass with the full network on the converged state (the
        # reference's BDF refine(), solver_3d.py:1056-1089), device time
        from prism3d_gb300.network import ChemistrySolverGPU
        net = ChemistrySolverGPU()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st_ref = s2.refine(network=net, mixed=True)
        t_ref = time.perf_counter() - t0
        net.close()
        refine = {"value": n / t_ref, "unit": "cells/s", "seconds": t_ref,
                  "unconverged_frac": float((st_ref != 0).mean()),
                  "sample": "every cell of the converged grid, host clock around "
                            "p3d_steady_refine (gather, network, scatter, thermal root)"}
    s2.close()
    h2d = dens.nbytes + 8 * (s.tables.pe_table.size + 3 * s.tables.n_bins + 60)
    d2h = sum(a.nbytes for a in outs)
    # plain FP64 path: full solve (and the mixed state's difference from it),
    # or a bounded sample of iterations
    s.reset()
    plain_full = args.plain_full or args.plain == "full" or (args.plain == "auto" and n <= 1 << 21)
    if plain_full:
        t0 = time.perf_counter()
        okp = s.run(max_iterations=4000, convergence_tol=args.tol, mixed=False, n_allow=n_allow,
                    w_chem=args.w_chem)
        tp = time.perf_counter() - t0
        plain = {"value": n / tp, "unit": "cells/s", "iterations": s.iterations,
                 "converged": bool(okp), "seconds": tp, "sample": "full solve"}
        # per-species difference of the mixed state (the e2e solve) from the
        # plain FP64 state, cells with the plain value above 1e-20
        err = {}
        for k, a in zip(STATE_KEYS, outs):
            b = s.get(k).ravel()
            a = a.ravel()
            m = np.abs(b) > 1e-20
            rel = np.abs(a - b)[m] / np.abs(b)[m]
            err[k] = {"frac_le_1e-6": float(np.mean(rel <= 1e-6)),
                      "frac_le_1e-4": float(np.mean(rel <= 1e-4)),
                      "median": float(np.median(rel)), "p99": float(np.percentile(rel, 99)),
                      "max": float(rel.max())}
        plain["mixed_vs_plain_rel_error"] = err
        accuracy = accuracy_block(outs, [s.get(k) for k in STATE_KEYS], chg_mixed > args.tol,
                                  s.get("change") > args.tol, n_allow)
    else:
        accuracy = None
        k = args.plain_iters
        t0 = time.perf_counter()
        s.run(max_iterations=k, convergence_tol=1e-300, mixed=False, n_allow=0, w_chem=args.w_chem)
        tp = time.perf_counter() - t0
        ms_it = 1e3 * tp / k
        est = n / (ms_it * 1e-3 * float(np.mean(iters)))
        plain = {"ms_per_iter": ms_it, "sample": f"first {k} outer iterations",
                 "value_est": est, "unit": "cells/s",
                 "note": "estimate = n_cells / (ms_per_iter x the mixed solve's iteration "
                         "count); --plain-full measures the full plain solve"}
    # rooflines, timed live from the 14th outer iteration of a fresh solve (the
    # state the per-cell FP64 count was measured on), every cell solved
    s.reset()
    s.run(max_iterations=13, convergence_tol=1e-300, mixed=True, n_allow=0, w_chem=args.w_chem)
    kt = kernel_times(s, reps=1)
    hbm, peak_kind = measured_peaks()
    fp64_peak = fp64_peak_tflops()
    # read the layers 2 n x_H2, n x_CO, family, ds and the columns at each
    # cell's last solve once; write N_H2, N_CO and the column-drift byte
    col_bytes = 58.0 * n
    col_gbs = col_bytes / (kt["columns_ms"] * 1e-3) / 1e9
    cell_tf = FP64_OPS_PER_CELL_SOLVE * n / (kt["cell_mixed_ms"] * 1e-3) / 1e12
    out = {
        "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (mixed)",
        "data": "synthetic (seeded Orion-Bar-like slab, prism3d_gb300/fields.py)",
        "config": {"workload": f"{args.workload}: {fields.WORKLOAD_DESC[args.workload]}, "
                               f"zeta={zeta:g}, 0.005 pc cells",
                   "n_cells": n, "tol": args.tol, "n_allow": n_allow, "w_chem": args.w_chem,
                   "outer_iterations": iters, "converged": oks,
                   "l2": "per-step state 0.6 GB > 126 MB L2 (no flush)",
                   "autotuned_cell_launch": {"threads": tuned[0], "blocks_per_sm": tuned[1],
                                             "ms_all_cells": tuned[2]},
                   "parallelism": f"replicas x{ws}"},
        "e2e": {"value": n / t_e2e, "unit": "cells/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "sample": "host clock: PDRSolverGPU from the host density (allocation, "
                          "uploads, ray march), run to convergence, 8 state fields read "
                          "back; grain tables (one-time host build) and tuned launch shape "
                          "reused"},
        "plain_fp64": plain,
        "mixed_vs_plain": (value / ws) / plain.get("value", plain.get("value_est")),
        "roofline": {"kernel": "ss_mark/chem/thermal_kernel<mixed> (~95% of the solve's device "
                               "time in the ncu launch list), every cell solved",
                     "bound": "fp64", "achieved": cell_tf, "peak": fp64_peak,
                     "unit": "TFLOP/s", "frac": cell_tf / fp64_peak,
                     "traffic": DRAM_BYTES_PER_CELL_SOLVE * n,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the "
                                       "chemistry and thermal launches of this pass at 128^3, "
                                       "per cell solved, times n (the mark kernel not included)",
                     "peak_source": "measured live: DFMA-chain kernel on this GPU",
                     "algorithmic_flops_per_launch": FP64_OPS_PER_CELL_SOLVE * n,
                     "per_unit": f"{FP64_OPS_PER_CELL_SOLVE:.0f} FP64 flops per cell solve "
                                 "(ncu DADD + DMUL + 2 DFMA counts of the two kernels)",
                     "fp32_flops_per_cell_solve": FP32_OPS_PER_CELL_SOLVE,
                     "counts_source": "ncu instruction and DRAM counters of this pass's "
                                      "chemistry and thermal launches (bench.py --profile "
                                      "kernels, 128^3)",
                     "fp64_pipe_active_ncu": FP64_PIPE_ACTIVE_NCU,
                     "counts_at_commit": COUNTS_AT_COMMIT["cell"]},
        "roofline_hbm": {"kernel": "ss_columns_kernel (3 axes x 2 directions, one launch per "
                                   "outer iteration)",
                         "bound": "hbm", "achieved": col_gbs, "peak": hbm, "unit": "GB/s",
                         "frac": col_gbs / hbm, "traffic": COLUMNS_DRAM_BYTES_PER_CELL * n,
                         "peak_source": peak_kind, "algorithmic_bytes_per_launch": col_bytes,
                         "note": "FP64-pipe bound (82% busy: 22 DADD per cell for the running "
                                 "sums), not HBM; traffic below the algorithmic bytes: the "
                                 "layers are partly L2-resident, the columns stay in L2 "
                                 "(ncu, bench.py --profile kernels); a full pass, where a "
                                 "mixed run's last iterations recompute only the tiles "
                                 "holding rewritten cells",
                         "counts_at_commit": COUNTS_AT_COMMIT["columns"]},
        "kernel_times_ms": kt,
        "fp64_net_heating_evals_per_cell_iter": float(np.mean(hist[:, 6]) / n),
        "gpu_launches": int(sum(launches)),
        "clocks": clk.summary(),
    }
    # column-density maps of the converged state (observation pipeline), host
    # clock around the C-ABI call (device work, small D2H of the maps)
    from prism3d_gb300.observations import column_density_maps
    s2b = PDRSolverGPU(dens, box, G0_external=g0, zeta_CR_0=zeta, nside_rt=nside, T_init=100.0)
    s2b.run(max_iterations=13, convergence_tol=1e-300, mixed=True, n_allow=0, w_chem=args.w_chem)
    tms = []
    for _ in range(4):
        t0 = time.perf_counter()
        column_density_maps(s2b, los_axis=2, inclination_deg=0.0)
        tms.append(time.perf_counter() - t0)
    s2b.close()
    tm = min(tms[1:])
    out["column_maps"] = {"ms": 1e3 * tm, "bytes_read": 40 * n,
                          "GB_per_s": 40 * n / tm / 1e9,
                          "note": "5 fields read once (n_H, x_H2, x_CO, x_C+, x_e), LOS = z, "
                                  "host clock around p3d_steady_column_maps"}
    out["rt_dropin"] = rt_dropin_bench(dens, g0, cell, nside, outs, hbm, peak_kind, fp64_peak,
                                       args.workload)
    if args.production and args.workload == "slab128":
        out["production_256"] = production_bench(args)
    out["cpu_baseline"] = cpu_baseline(args, dens, g0, nside, zeta, cell, float(np.mean(iters)))
    # per outer iteration (cell updates per second): the comparison that needs
    # no assumption about how many iterations the reference would take
    it_cpu = out["cpu_baseline"].pop("seconds_per_iteration")
    out["per_iteration"] = {
        "unit": "cell updates/s (cells x outer iterations / time)",
        "mixed_gpu": n * float(np.mean(iters)) / (t_step / ws),
        "plain_gpu": (n * plain["iterations"] / plain["seconds"]) if "iterations" in plain
        else n / (plain["ms_per_iter"] * 1e-3),
        "reference_cpu_port": n / it_cpu}
    if args.network_cells > 0:
        out["network"] = network_bench(args)
        out["network"]["refine_pass"] = refine
    if accuracy is not None:
        # last in the line, so the end of the output carries it
        out["accuracy"] = accuracy
        out["accuracy_ok"] = accuracy.pop("ok")
    return out


def production_bench(args):
    """The production-size grid: 256^3 cored slab (tanh ramp 1e3 -> 3e5 x
    log-normal 1.2 with Gaussian cores of 1e6, zeta 5e-16, 48 rays), one
    mixed-precision solve on the device clock; and the per-species difference
    of mixed from plain FP64 on a 64^3 subvolume of the same density (the
    corner cube at the highest x, where the cores sit), both solved as grids
    of their own."""
    import numpy as np

    from prism3d_gb300 import fields
    from prism3d_gb300.solver import PDRSolverGPU
    dens, g0, nside, zeta, cell = fields.workload("slab256", seed=1)
    n = dens.size
    s = PDRSolverGPU(dens, cell * dens.shape[0], G0_external=g0, zeta_CR_0=zeta,
                     nside_rt=nside, T_init=100.0)
    tuned = s.autotune()
    n_allow = max(8, int(1e-5 * n))
    ok = s.run(max_iterations=4000, convergence_tol=args.tol, mixed=True, n_allow=n_allow,
               w_chem=args.w_chem)
    ms = s.elapsed_ms()
    res = {"workload": fields.WORKLOAD_DESC["slab256"], "n_cells": n, "converged": bool(ok),
           "outer_iterations": s.iterations, "seconds": ms * 1e-3, "cells_per_s": n / (ms * 1e-3),
           "autotuned_cell_launch": list(tuned[:2])}
    kt = kernel_times(s, reps=1)
    res["columns_ms"] = kt["columns_ms"]
    s.close()
    sub = np.ascontiguousarray(dens[-64:, -64:, -64:])
    st = {}
    for mixed in (True, False):
        q = PDRSolverGPU(sub, cell * 64, G0_external=g0, zeta_CR_0=zeta, nside_rt=nside,
                         T_init=100.0)
        q.run(max_iterations=4000, convergence_tol=args.tol, mixed=mixed,
              n_allow=max(8, int(1e-5 * sub.size)), w_chem=args.w_chem)
        st[mixed] = {k: q.get(k) for k in STATE_KEYS + ("change",)}
        q.close()
    err = {}
    for k in STATE_KEYS:
        a, b = st[True][k].ravel(), st[False][k].ravel()
        m = np.abs(b) > 1e-20
        rel = np.abs(a - b)[m] / np.abs(b)[m]
        err[k] = {"frac_le_1e-6": float(np.mean(rel <= 1e-6)), "p99": float(np.quantile(rel, 0.99)),
                  "max": float(rel.max())}
    res["subvolume_64_mixed_vs_plain"] = err
    acc = accuracy_block([st[True][k] for k in STATE_KEYS], [st[False][k] for k in STATE_KEYS],
                         st[True]["change"] > args.tol, st[False]["change"] > args.tol,
                         max(8, int(1e-5 * sub.size)))
    res["subvolume_64_accuracy"] = {k: acc[k] for k in ("cells_beyond", "cells_beyond_settled",
                                                        "moving", "n_allow", "ok")}
    return res


def rt_dropin_bench(dens, g0, cell, nside, state, hbm, peak_kind, fp64_peak, workload):
    """The drop-in FUV transfer (compute_fuv_field_3d, the call the
    reference's solver makes every outer iteration) on the converged state:
    device tensors on torch's stream (CUDA events), and from NumPy arrays
    through the C ABI (host clock, copies included)."""
    import numpy as np
    import torch

    from prism3d_gb300.core import compute_fuv_field_3d
    xh2, xco = np.ascontiguousarray(state[2]), np.ascontiguousarray(state[5])
    n = dens.size
    dd, dh2, dco = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (dens, xh2, xco))
    for _ in range(2):
        compute_fuv_field_3d(dd, g0, cell, dh2, dco, nside)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    e0.record()
    for _ in range(reps):
        compute_fuv_field_3d(dd, g0, cell, dh2, dco, nside)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    t0 = time.perf_counter()
    for _ in range(2):
        compute_fuv_field_3d(dens, g0, cell, xh2, xco, nside)
    t_host = (time.perf_counter() - t0) / 2
    gbs = 64.0 * n / (ms * 1e-3) / 1e9
    res = {"ms": ms, "cells_per_s": n / (ms * 1e-3), "e2e_cells_per_s": n / t_host,
           "e2e_h2d_bytes": 24 * n, "e2e_d2h_bytes": 44 * n,
           "hbm": {"achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                   "peak_source": peak_kind,
                   "per_unit": "64 B per cell (read n_H, x_H2, x_CO; write G0, A_V, N_H, N_H2, "
                               "N_CO)"},
           "rays": 12 * nside * nside}
    if workload in RT_FP64_OPS_PER_CELL and nside == 2:
        tf = RT_FP64_OPS_PER_CELL[workload] * n / (ms * 1e-3) / 1e12
        res["roofline"] = {"bound": "fp64", "achieved": tf, "peak": fp64_peak, "unit": "TFLOP/s",
                           "frac": tf / fp64_peak, "peak_source": "measured live: DFMA-chain "
                           "kernel on this GPU", "traffic": RT_DRAM_BYTES_PER_CELL[workload] * n,
                           "per_unit": f"{RT_FP64_OPS_PER_CELL[workload]:.0f} FP64 flops per cell "
                                       "(walk + merge, 48 rays; ncu counts, "
                                       "bench.py --profile rt)",
                           "counts_at_commit": COUNTS_AT_COMMIT["rt"]}
    return res


def network_bench(args):
    """Full 31-species network steady state (the reference's per-cell BDF
    solve, prism3d/chemistry/solver.py:145-225) on seeded cells: device time
    of the mixed and FP64 kernels, the host-buffer C ABI end to end, and the
    CPU oracle on a bounded sample."""
    import numpy as np
    import torch

    from prism3d_gb300 import fields
    from prism3d_gb300.network import ChemistrySolverGPU

    n = args.network_cells
    net = ChemistrySolverGPU()
    cond = fields.network_cells(n, seed=11)
    x0 = net.default_initial_batch(cond[:, 2], cond[:, 3])
    dc = torch.from_numpy(cond).cuda()
    dx0 = torch.from_numpy(x0).cuda()
    res = {"cells": n, "workload": "seeded cells over the PDR parameter span "
           "(prism3d_gb300/fields.py:network_cells), the reference's initial abundances",
           "rtol": 1e-8, "max_iter": 300}
    for mixed in (True, False):
        for rep in range(2):  # one warm-up, one timed
            dx = dx0.clone()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            st, it = net.solve_steady_state_batch(dc, dx, mixed=mixed, post=True,
                                                  return_iters=True)
            e1.record()
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        st, it = st.cpu().numpy(), it.cpu().numpy()
        res["mixed" if mixed else "fp64"] = {
            "value": n / (ms * 1e-3), "unit": "cells/s", "ms": ms,
            "newton_iters_mean": float(it.mean()), "unconverged_frac": float((st != 0).mean())}
    t0 = time.perf_counter()
    xh = x0.copy()
    net.solve_steady_state_batch(cond, xh, mixed=True, post=True)
    t = time.perf_counter() - t0
    res["e2e"] = {"value": n / t, "unit": "cells/s", "h2d_bytes": int(cond.nbytes + x0.nbytes),
                  "d2h_bytes": int(x0.nbytes + 8 * n)}
    net.close()
    # CPU oracle (NumPy restatement of the same method, vectorised over cells)
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from oracle import network as ON
    m = min(args.network_cpu_sample, n)
    t0 = time.perf_counter()
    ON.solve_steady_state(ON.load(), x0[:m], cond[:m])
    t = time.perf_counter() - t0
    res["cpu_baseline"] = {"value": m / t, "unit": "cells/s", "cores": 1, "kind": "port",
                           "sample": f"first {m} cells, NumPy oracle"}
    return res


# Per-cell counts of the launches bench.py times for its rooflines, from ncu
# on `bench.py --profile kernels` / `--profile rt` at 128^3 (2,097,152
# cells, one kernel per capture, --clock-control none):
# FP64 flops (DFMA = 2, DADD / DMUL = 1) per cell solve of the mixed
# chemistry (1,093) and thermal (1,043) kernels on the 14th outer iteration,
# every cell solved with exact roots, and their FP32 flops (723 + 5,978);
# DRAM bytes of the two launches (read + write: 328.5 + 212.6 and 536.3 +
# 301.1 MB): the state is streamed once per solve, so the traffic scales
# with the cells solved.
FP64_OPS_PER_CELL_SOLVE = 1092.9 + 1042.6
FP32_OPS_PER_CELL_SOLVE = 723.0 + 5977.7
DRAM_BYTES_PER_CELL_SOLVE = (328.5 + 212.6 + 536.3 + 301.1) * 1e6 / 2097152
FP64_PIPE_ACTIVE_NCU = ("85% (chemistry), 72% (thermal): the pipe also runs FP64 compares, "
                        "min/max and FP32<->FP64 conversions; the thermal kernel's remaining "
                        "time is latency of divergent root paths")
# columns launch (a full pass): FP64-pipe bound (82% busy), 29 FP64 flops
# per cell; DRAM per launch (read + write) with the chemistry's layers partly
# L2-resident
COLUMNS_DRAM_BYTES_PER_CELL = (82.1 + 13.5) * 1e6 / 2097152
# drop-in ray march (walk + merge, 48 rays) at 128^3: FP64 flops per cell
# and DRAM bytes per cell of the two launches
RT_FP64_OPS_PER_CELL = {"slab128": 684.0 + 12.0}
RT_DRAM_BYTES_PER_CELL = {"slab128": (233.6 + 460.8 + 344.5 + 74.4) * 1e6 / 2097152}
# the source revision each capture above ran on (none of the captured
# kernels has changed since)
COUNTS_AT_COMMIT = {"cell": {"ss_chem_kernel": "4093bfe", "ss_thermal_kernel": "95ae15a"},
                    "columns": "e85e9b0", "rt": "e85e9b0"}
STATE_KEYS = ("T_gas", "x_HI", "x_H2", "x_Cp", "x_C", "x_CO", "x_O", "x_e")


def accuracy_block(mixed, plain, moving_mixed, moving_plain, n_allow):
    """Mixed-precision steady state against the plain FP64 one, cell by cell:
    per field the fraction of cells within the tolerance (1e-6 relative for
    the abundances, which are relative to n_H, counted where the plain value
    is above 1e-20; 1e-4 for T_gas) and the largest relative difference.
    A solve converges when at most n_allow cells still change by more than
    tol per iteration; those cells (moving_*: the per-cell change of the
    last solve above tol) have not settled in one solve or the other and are
    counted apart: cells_beyond counts every cell with a field beyond its
    tolerance, cells_beyond_settled those among the settled cells.
    ok: no settled cell beyond tolerance, and each solve left at most
    n_allow cells moving."""
    import numpy as np
    fields = {}
    beyond = None
    for k, a, b in zip(STATE_KEYS, mixed, plain):
        a, b = np.ravel(a), np.ravel(b)
        m = np.abs(b) > 1e-20
        rel = np.zeros(a.shape)
        rel[m] = np.abs(a - b)[m] / np.abs(b)[m]
        tol = 1e-4 if k == "T_gas" else 1e-6
        bad = rel > tol
        beyond = bad if beyond is None else (beyond | bad)
        fields[k] = [round(float(np.mean(~bad)), 7), float(rel.max())]
    moving = np.ravel(moving_mixed) | np.ravel(moving_plain)
    settled_bad = int(np.sum(beyond & ~moving))
    return {"tol": {"species": 1e-6, "T_gas": 1e-4}, "within_and_max": fields,
            "cells_beyond": int(beyond.sum()), "cells_beyond_settled": settled_bad,
            "moving": [int(np.sum(moving_mixed)), int(np.sum(moving_plain))],
            "n_allow": int(n_allow), "n_cells": int(beyond.size),
            "ok": bool(settled_bad == 0 and np.sum(moving_mixed) <= n_allow
                       and np.sum(moving_plain) <= n_allow)}


def fp64_peak_tflops():
    import ctypes

    from prism3d_gb300 import _lib as L
    v = ctypes.c_double(0.0)
    L.call("p3d_fp64_peak_tflops", ctypes.byref(v))
    return float(v.value)


def kernel_times(s, reps=10):
    """Mean launch time of the per-iteration kernels on the current state."""
    import ctypes

    from prism3d_gb300 import _lib as L
    ms = (ctypes.c_double * 4)()
    L.call("p3d_steady_kernel_times", s._h, reps, ctypes.cast(ms, L._D))
    return {"columns_ms": ms[0], "reduce_ms": ms[1], "cell_mixed_ms": ms[2],
            "cell_plain_ms": ms[3]}


def cpu_baseline(args, dens, g0, nside, zeta, cell, gpu_iters):
    """One reference outer iteration on the CPU oracle, all host threads."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    O.reference_run(dens, g0, cell, nside=nside, zeta0=zeta, T_init=100.0, n_iter=1,
                    n_substeps=200)
    t_it = time.perf_counter() - t0
    return {"value": dens.size / (t_it * gpu_iters), "unit": "cells/s",
            "cores": os.cpu_count(), "kind": "port", "seconds_per_iteration": t_it,
            "sample": f"one reference outer iteration on the full {dens.shape} grid "
                      f"({t_it:.2f} s; C oracle with OpenMP + NumPy ray march), "
                      f"scaled by the GPU solve's {gpu_iters:.0f} outer iterations"}


def run_reference(args, ws, rank):
    if rank != 0:
        return None
    import numpy as np

    from oracle import oracle as O
    from prism3d_gb300 import fields
    dens, g0, nside, zeta, cell = fields.workload(args.workload, seed=1)
    n = dens.size
    iters = args.ref_iters
    for _ in range(args.warmup):
        O.reference_run(dens[:16], g0, cell, nside=nside, zeta0=zeta, T_init=100.0, n_iter=1)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.reference_run(dens, g0, cell, nside=nside, zeta0=zeta, T_init=100.0, n_iter=1,
                        n_substeps=200)
        times.append(time.perf_counter() - t0)
    t_it = float(np.mean(times))
    value = n / (t_it * iters)
    return {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_it * iters,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Orion-Bar-like slab)", "impl": "reference",
            "config": {"workload": f"{args.workload}: {fields.WORKLOAD_DESC[args.workload]}, "
                                   f"zeta={zeta:g}, 0.005 pc cells; converged cells/s = one "
                                   f"measured reference outer iteration x outer_iterations_assumed "
                                   f"= {iters} (the GPU solve's count: the reference's own run() "
                                   f"does not converge)",
                       "n_cells": n, "outer_iterations_assumed": iters},
            "per_iteration": {"unit": "cell updates/s (cells x outer iterations / time)",
                              "reference_cpu_port": n / t_it,
                              "seconds_per_iteration": t_it},
            "cpu_baseline": {"value": value, "unit": "cells/s", "cores": os.cpu_count(),
                             "kind": "port",
                             "sample": f"one reference outer iteration per step on the full "
                                       f"grid ({t_it:.2f} s), x {iters} iterations"},
            "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def profile_run(args):
    """Short, deterministic runs for ncu (no autotune, no comparison solves):
    the launches the bench line times, with nothing else around them."""
    import torch

    from prism3d_gb300 import fields
    from prism3d_gb300.solver import PDRSolverGPU
    torch.cuda.set_device(0)
    dens, g0, nside, zeta, cell = fields.workload(args.workload, seed=1)
    n = dens.size
    s = PDRSolverGPU(dens, cell * dens.shape[0], G0_external=g0, zeta_CR_0=zeta, nside_rt=nside,
                     T_init=100.0)
    t, b = (int(v) for v in args.launch.split(","))
    s.set_launch(t, b)
    out = {"profile": args.profile, "workload": args.workload, "n_cells": n, "launch": [t, b]}
    if args.profile == "rt":
        # the drop-in ray march on device tensors (its work depends on the
        # geometry, not on the abundances)
        from prism3d_gb300.core import compute_fuv_field_3d
        dd = torch.from_numpy(dens).cuda()
        dh2 = torch.full_like(dd, 0.25)
        dco = torch.full_like(dd, 1e-4)
        for _ in range(2):
            compute_fuv_field_3d(dd, g0, cell, dh2, dco, nside)
        torch.cuda.synchronize()
        out["rays"] = 12 * nside * nside
    elif args.profile == "solve":
        s.reset()
        ok = s.run(max_iterations=4000, convergence_tol=args.tol, mixed=True,
                   n_allow=max(8, int(1e-5 * n)), w_chem=args.w_chem)
        h = s.convergence_history()
        out.update({"converged": bool(ok), "outer_iterations": s.iterations,
                    "ms": s.elapsed_ms(), "gpu_launches": s.launch_count(),
                    "cell_solves_per_cell": float(h[:, 8].sum() / n)})
    else:
        s.run(max_iterations=13, convergence_tol=1e-300, mixed=True, n_allow=0,
              w_chem=args.w_chem)
        out["kernel_times_ms"] = kernel_times(s, reps=1)
    s.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="slab128")
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--w-chem", type=float, default=0.1,
                    help="abundance damping (the reference uses 0.5)")
    ap.add_argument("--plain", default="auto", choices=["auto", "full", "estimate"],
                    help="plain FP64 comparison: a full solve (auto: up to 2^21 cells) or a "
                         "per-iteration sample")
    ap.add_argument("--plain-full", action="store_true", help="same as --plain full")
    ap.add_argument("--plain-iters", type=int, default=20)
    ap.add_argument("--ref-iters", type=int, default=440,
                    help="outer iterations the reference arm is scaled by (the GPU solve of "
                         "the 128^3 slab takes 440)")
    ap.add_argument("--network-cells", type=int, default=1 << 20,
                    help="cells of the full-network measurement (0: skip)")
    ap.add_argument("--network-cpu-sample", type=int, default=2048)
    ap.add_argument("--production", type=int, default=1,
                    help="1: also solve the 256^3 production grid (one mixed solve) and "
                         "compare mixed with plain FP64 on a 64^3 subvolume")
    ap.add_argument("--profile", default="", choices=["", "solve", "kernels", "rt"],
                    help="a short run for ncu instead of the bench line: 'solve' = one mixed "
                         "solve from the initial state (the launch list); 'kernels' = 13 mixed "
                         "iterations, then one p3d_steady_kernel_times pass (the per-kernel "
                         "counters: its mixed chemistry and thermal launches are the 14th of "
                         "their kernels, the plain ones follow); 'rt' = two drop-in "
                         "compute_fuv_field_3d calls after the solver's own ray march")
    ap.add_argument("--launch", default="128,8",
                    help="with --profile: per-cell launch shape (threads,blocks per SM) in "
                         "place of the autotuner's choice")
    args = ap.parse_args()
    ws, rank, local = _dist()
    if args.profile:
        print(json.dumps(profile_run(args)))
        return
    if ws > 1:
        import torch
        import torch.distributed as dist
        if args.impl == "gb300":
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    if args.impl == "reference":
        out = run_reference(args, ws, rank)
    else:
        out = run_gb300(args, ws, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
