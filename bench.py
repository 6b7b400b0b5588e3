#!/usr/bin/env python
"""Benchmark of FFEA's per-timestep blob update on GB300.

Workload (one "step" = one blob time step): a 40x40x40-cell Kuhn-split cube
of side 200 nm (384,000 linear tets, 68,921 vertex nodes), seeded +-5% interior
jitter, density 1500 kg/m^3, G = 5.7e8 Pa, K = 2.2e9 Pa, shear and bulk
viscosity 1e-3 Pa s; NoMassCGSolver with CG tolerance 1e-10, dt = 1e-12 s,
kT = 4.11e-21 J (thermal noise on, MRG32k3a stream 12345 x 6). Inputs are
seeded synthetic meshes; there is no dataset.

A second workload (`--workload batch`, and the "batched" object of the default line) is the
replica ensemble: 256 Kuhn cubes with cells per side log-uniform in [8, 32] (seeded), per-blob
G ~ U[1e8, 1e9] Pa and K = 3.9 G, all advanced by one graph-captured step (mixed precision).

The "scale" object runs the 64^3-cell cube (1,572,864 tets), CG_nomass and mass-lumped, mixed
against FP64. The "adjoint" object times the gradient of a 200-step window of a 20^3-cell cube with lognormal
per-element moduli (checkpoints every 20 steps): seconds per step of gradient and its cost relative
to the forward window.

Metric: node-steps/s = vertex nodes x steps / time (whole job, all GPUs).
Default arm: the mixed-precision GPU path (headline), with the plain FP64
GPU path timed beside it. `--impl reference` times the reference algorithm on
the host cores instead: the oracle's C restatement with OpenMP (kind "port"),
because the reference's own sources do not travel to the benchmark machine, so
its compiled build (oracle/_ref) exists only where the sources are.

Timing: W untimed warm-up steps, then K steps each timed by CUDA events on
the blob's stream, with 256 MiB of scratch written before every step outside
the timed window (cold L2 for every step); max over ranks. Under torchrun each
rank runs an independent replica on its own GPU (replicas only: a single blob
does not shard), so the job's value is the sum of replica throughputs.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_CELLS, SIDE = 40, 200.0
PHYS = dict(solver="CG_nomass", dt=1e-12, kT=4.11e-21, epsilon=1e-10, max_iterations_cg=10000, calc_noise=1,
            calc_stokes=0)
FLUSH_BYTES = 256 << 20
MESO_LENGTH = 1.7e-10
MESO_FORCE = 2.4364705882352941e-11


def workload_config(n: int, precision: str) -> dict:
    from ffea_ci_demo_gb300.mesh import counts

    c = counts(n)
    return {"workload": f"kuhn-cube-{n}: {c['T']} tets, {c['N']} nodes, NoMassCG eps=1e-10, dt=1e-12 s, "
                        f"kT=4.11e-21 J", "cells_per_side": n, "tets": c["T"], "nodes": c["N"],
            "matrix_nnz": c["nnz_linear"], "solver": "CG_nomass", "precision": precision,
            "l2": "flushed before every timed step (256 MiB scratch write)"}


def rank_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Replicas:
    """The ranks of a multi-GPU run: one independent replica of the workload per rank (a blob does not shard),
    host-side barriers and the max over ranks of a timing through gloo (no collective touches the data path).
    A run's throughput is the units all ranks processed divided by the slowest rank's time."""

    def __init__(self, world_size: int):
        self.ws = world_size
        self.dist = None
        if world_size > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self) -> None:
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if not self.dist:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def throughput(self, units_per_rank: float, seconds: float) -> float:
        return self.ws * units_per_rank / self.max(seconds)

    def close(self) -> None:
        if self.dist:
            self.dist.destroy_process_group()
            self.dist = None


def pick_device(local: int) -> str:
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    phys = vis.split(",")[local] if vis else str(local)
    os.environ["CUDA_VISIBLE_DEVICES"] = phys
    return phys


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: str):
        self.gpu, self.lines, self.proc = gpu, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", self.gpu], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak() -> tuple[float, str]:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled(name: str, key: str):
    """A figure from a committed ncu summary (profiles/<name>.txt, `key = value` lines), or None."""
    path = os.path.join(ROOT, "profiles", name + ".txt")
    try:
        for ln in open(path):
            if ln.split("=")[0].strip() == key:
                return float(ln.split("=")[1].split()[0])
    except (OSError, ValueError, IndexError):
        pass
    return None


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith(("model name", "cpu part")):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


_PINNED = []


def host_array(shape):
    """A float64 host array in page-locked memory (torch's pinned allocator) for the end-to-end runs, or
    ordinary memory if that is not available; returns the array and which it is."""
    import numpy as np
    try:
        import torch

        t = torch.empty(shape, dtype=torch.float64, pin_memory=True)
        _PINNED.append(t)  # the array below is a view of t's memory: keep t alive
        return t.numpy(), "pinned"
    except Exception:  # noqa: BLE001 - any failure to pin falls back to pageable memory
        return np.empty(shape), "pageable"


def cg_bytes_per_iteration(n: int, p: int) -> float:
    """Compulsory bytes of one CG iteration by the per-unit model: nnz (p + 4) + (R + 1) 4 + 8 R p."""
    from ffea_ci_demo_gb300.mesh import counts

    c = counts(n)
    R = 3 * c["N"]
    return c["nnz_linear"] * (p + 4) + (R + 1) * 4 + 8 * R * p


def cg_format_bytes_per_iteration(blocks: int, nodes: int, p: int) -> float:
    """Bytes the SELL 3x3-block matrix actually holds per SpMV (values + block columns + row data)
    plus eight passes over padded 4-wide vectors."""
    return blocks * (9 * p + 4) + nodes * 8 + 8 * nodes * 4 * p


def cheb_pass_bytes(n: int, p: int) -> float:
    """One extra matrix pass of the Chebyshev preconditioner by the per-unit model's terms: the matrix
    (nnz (p + 4) + (R + 1) 4) and two vector passes (2 R p)."""
    from ffea_ci_demo_gb300.mesh import counts

    c = counts(n)
    R = 3 * c["N"]
    return c["nnz_linear"] * (p + 4) + (R + 1) * 4 + 2 * R * p


def masslumped_bytes_per_step(n: int, p: int) -> float:
    """Compulsory bytes of one mass-lumped step by the per-unit model:
    T (16 + 14 p + 16) + N 48 + 2 (12 T p) + 16 T + 4 (N + 1) + N (24 + 8 + 96)."""
    from ffea_ci_demo_gb300.mesh import counts

    c = counts(n)
    T, N = c["T"], c["N"]
    return T * (16 + 14 * p + 16) + N * 48 + 2 * 12 * T * p + 16 * T + 4 * (N + 1) + N * (24 + 8 + 96)


def run_gpu_arm(args, ws, rank, local) -> dict | None:
    import numpy as np

    from ffea_ci_demo_gb300 import build, lib
    from ffea_ci_demo_gb300.mesh import apply_shear, counts, kuhn_cube

    ranks = Replicas(ws)
    barrier, max_over_ranks = ranks.barrier, ranks.max
    build.build()
    n = args.cells
    mesh = kuhn_cube(n, side=SIDE * n / N_CELLS, seed=12345)
    N = counts(n)["N"]
    gpu = os.environ.get("CUDA_VISIBLE_DEVICES", "0")

    out = {}
    for prec in (["mixed", "fp64"] if args.precision == "both" else [args.precision]):
        blob = lib.Blob(mesh, precision=prec, **PHYS)
        blob.update(args.warmup)
        # the mixed CG's preconditioner after warm-up (the first solve is Jacobi's, the second the polynomial's
        # trial): each CG iteration applies the matrix 1 + degree times
        deg, lmax = blob.cg_preconditioner()
        it0 = blob.cg_iterations()[1]
        l0 = lib.launch_count()
        barrier()
        steps = args.steps if prec == "mixed" or args.precision != "both" else max(3, args.steps // 4)
        with Clocks(gpu) as clk:
            t = blob.update_timed(steps, FLUSH_BYTES)
        barrier()
        launches = lib.launch_count() - l0
        iters = blob.cg_iterations()[1] - it0
        ms = max_over_ranks(t["ms"])
        nl, ne, nb = blob.sizes()
        out[prec] = {"ms": ms, "steps": steps, "value": ws * N * steps / (ms / 1e3), "phase_ms": t["phase_ms"],
                     "cg_iters_per_step": iters / steps, "launches": launches, "clocks": clk.summary(),
                     "blocks": nb, "cg_poly": deg, "lambda_max": lmax, "cg_kernel": blob.cg_kernel()}
        if prec == args.headline:
            # end to end through the C ABI: every node's host position (the reference's layout, midpoints
            # included, in pinned host memory) in, one step, every position out
            pos_host, mem_kind = host_array((blob.n_nodes, 3))
            blob.pos(out=pos_host)
            k = max(3, steps // 2)
            barrier()
            t0 = time.perf_counter()
            for _ in range(k):
                blob.set_state(pos=pos_host)
                blob.update(1)
                blob.pos(out=pos_host)
            t1 = time.perf_counter()
            barrier()
            e2e_s = max_over_ranks(t1 - t0)
            nbytes = 24 * blob.n_nodes
            out[prec]["e2e"] = {"value": ws * N * k / e2e_s, "unit": "node-steps/s", "h2d_bytes_per_step": nbytes,
                                "d2h_bytes_per_step": nbytes, "steps": k, "host_memory": mem_kind}
        blob.close()
    # kT = 0 error of the mixed path (the timed arithmetic: same kernel, same preconditioner) against the FP64
    # path from the same initial shear, after error_steps steps; the stated bound is 1e-5 after 1000 steps
    if args.precision == "both" and args.error_steps > 0:
        p0 = apply_shear(mesh, 0.02, seed=3) * (mesh.scale / MESO_LENGTH)
        res, how = {}, {}
        for prec in ("fp64", "mixed"):
            b = lib.Blob(mesh, precision=prec, **dict(PHYS, kT=0.0, calc_noise=0))
            b.set_state(pos=p0)
            b.update(min(2, args.error_steps))
            how[prec] = (b.cg_kernel(), b.cg_preconditioner()[0])
            b.update(args.error_steps - min(2, args.error_steps))
            res[prec] = b.pos()
            b.close()
        d = np.abs(res["mixed"] - res["fp64"]).max() / np.abs(res["fp64"] - p0).max()
        out["error"] = {"kT0_steps": args.error_steps, "max_abs_disp_err_rel_to_max_disp": float(d),
                        "bound": 1e-5, "within_bound": bool(d <= 1e-5),
                        "mixed_arithmetic": f"{how['mixed'][0]}, chebyshev degree {how['mixed'][1]}"
                        if how["mixed"][1] else f"{how['mixed'][0]}, jacobi",
                        "reference": "FP64 GPU path (bit-exact element math vs the reference; CG to rounding; "
                                     "tied to the oracle at this size by tests/test_headline.py)"}
    # kT > 0: both paths from the same state with the same noise stream; RMS position difference against the
    # RMS displacement, and each path's mean strain energy against equipartition, (3N - 6) kT / 2
    if args.precision == "both" and args.kt_steps > 0:
        res = {}
        for prec in ("fp64", "mixed"):
            b = lib.Blob(mesh, precision=prec, **PHYS)
            x0 = b.pos()
            se = []
            for _ in range(args.kt_steps // 10):
                b.update(10)
                se.append(b.measurements()["strain_energy"])
            res[prec] = (b.pos(), np.array(se), x0)
            b.close()
        xf, xm, x0 = res["fp64"][0], res["mixed"][0], res["fp64"][2]
        rms = float(np.sqrt(np.mean((xm - xf) ** 2)) / np.sqrt(np.mean((xf - x0) ** 2)))
        want = (3 * N - 6) / 2.0  # kT in meso units is PHYS kT / mesoDimensions::Energy
        want *= PHYS["kT"] / 4.141945559999999e-21
        half = lambda a: a[len(a) // 2:]
        out.setdefault("error", {})["kT"] = {
            "steps": args.kt_steps, "rms_pos_diff_rel_to_rms_disp": rms,
            "equipartition_dev_fp64": float(half(res["fp64"][1]).mean() / want - 1),
            "equipartition_dev_mixed": float(half(res["mixed"][1]).mean() / want - 1),
            "note": "strain energy averaged over the second half of the run, sampled every 10 steps; at dt = 1e-12 s "
                    "the explicit Euler step is comparable to the stiffest modes' relaxation time, so both paths "
                    "(and the reference's algorithm) sit the same amount above equipartition"}
    ranks.close()
    return out if rank == 0 else None


def batch_bytes_per_iteration(cells: int, p: int) -> tuple[float, float]:
    """Per-unit model bytes and SELL-format bytes of one CG iteration of one n^3-cell blob."""
    from ffea_ci_demo_gb300.mesh import counts

    c = counts(cells)
    R = 3 * c["N"]
    model = c["nnz_linear"] * (p + 4) + (R + 1) * 4 + 8 * R * p
    fmt = c["nnz_blocks"] * (9 * p + 4) + c["N"] * 8 + 8 * c["N"] * 4 * p
    return float(model), float(fmt)


def run_batch(args, ws, rank=0, ranks=None) -> dict:
    """Configuration 2: the replica ensemble, all blobs advanced by one graph-captured step. With ws ranks, the
    ensemble is split over them by element count (ffea_ci_demo_gb300.shard) and each rank steps a batch of its own
    blobs; the time is the slowest rank's and the throughput counts every rank's nodes (strong scaling: the
    ensemble is fixed)."""
    from ffea_ci_demo_gb300 import build, lib
    from ffea_ci_demo_gb300.mesh import ensemble, ensemble_cells
    from ffea_ci_demo_gb300.shard import partition_by_elements

    build.build()
    cells_all = [int(n) for n in ensemble_cells(args.blobs)]
    meshes_all = ensemble(args.blobs)
    mine = partition_by_elements([m.n_elem for m in meshes_all], ws)[rank] if ws > 1 else list(range(args.blobs))
    meshes = [meshes_all[b] for b in mine]
    cells = [cells_all[b] for b in mine]
    nodes_all = sum(m.n_linear for m in meshes_all)
    barrier = ranks.barrier if ranks else (lambda: None)
    max_over = ranks.max if ranks else (lambda x: x)
    bt = lib.Batch(meshes, **{k: v for k, v in PHYS.items() if k != "solver"})
    sz = bt.sizes()
    bt.update(args.warmup)
    tuned_ms = None
    if args.no_tune:
        bt.set_config(args.cg_threads, args.tpn)
    else:
        tuned_ms = bt.tune(1)
    cfg = bt.config()
    tot0 = bt.cg_iterations()[1]
    l0 = lib.launch_count()
    k = args.steps
    barrier()
    with Clocks(os.environ.get("CUDA_VISIBLE_DEVICES", "0")) as clk:
        t = bt.update_timed(k, FLUSH_BYTES, cg=True)
    barrier()
    t_all = max_over(t["ms"])
    launches = lib.launch_count() - l0
    last, tot1 = bt.cg_iterations()
    iters_per_step = (tot1 - tot0) / k
    # per-blob iterations of the timed steps, estimated from the last step's split of the total
    scale = iters_per_step / max(1, int(last.sum()))
    model = fmt = 0.0
    for n, it in zip(cells, last.tolist()):
        mb, fb = batch_bytes_per_iteration(n, 4)
        model += it * scale * mb
        fmt += it * scale * fb
    ms = t["ms"] / k
    cg_ms = t["cg_ms"] / k
    peak, peak_kind = measured_peak()
    out = {"workload": f"ensemble of {args.blobs} Kuhn cubes, cells per side log-uniform in [8,32] (seeded), "
                       f"G ~ U[1e8,1e9] Pa, K = 3.9 G; NoMassCG eps=1e-10, dt=1e-12 s, kT=4.11e-21 J, mixed",
           "blobs": len(meshes_all), "nodes": nodes_all, "tets": sum(m.n_elem for m in meshes_all),
           "matrix_blocks_this_rank": sz["blocks"],
           "value": nodes_all * k / (t_all / 1e3), "unit": "node-steps/s", "ms_per_step": t_all / k, "steps": k,
           "blobs_this_rank": len(mine), "nodes_this_rank": sz["nodes"],
           "warmup": args.warmup, "cg_iters_per_step_all_blobs": iters_per_step,
           "cg_iters_per_blob": {"min": int(last.min()), "mean": float(last.mean()), "max": int(last.max())},
           "launch_config": cfg, "tuned_best_solve_ms": tuned_ms, "gpu_launches": launches,
           "clocks": clk.summary(),
           "roofline": {"bound": "hbm", "kernel": "cg_batch_kernel",
                        "achieved": fmt / (cg_ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": fmt / (cg_ms / 1e3) / 1e9 / peak, "peak_source": peak_kind,
                        "ms_per_launch": cg_ms,
                        "frac_over_whole_step": fmt / (ms / 1e3) / 1e9 / peak,
                        "bytes": "SELL format per CG iteration of each blob x its iterations",
                        "traffic": (fmt * ratio) if (ratio := profiled("cg_batch_kernel_ensemble64",
                                                                       "dram_bytes_per_format_byte")) else None,
                        "traffic_note": "DRAM bytes per step scaled by format bytes from the ncu capture of a timed "
                                        "launch of the 64-blob ensemble (profiles/cg_batch_kernel_ensemble64.txt)",
                        # the captured launch's DRAM bytes over its duration, against the measured copy peak
                        "dram_frac_cg_kernel": profiled("cg_batch_kernel_ensemble64", "dram_gbs") / peak
                        if profiled("cg_batch_kernel_ensemble64", "dram_gbs") else None,
                        "bytes_per_step_format_cg": fmt, "bytes_per_step_model_cg": model,
                        "model_equiv_gbs": model / (ms / 1e3) / 1e9}}
    if ws > 1:
        out["sharding"] = {"ranks": ws, "split": "element counts balanced, longest first (ffea_ci_demo_gb300.shard)",
                           "collective": "none on the data path (gloo barrier and max of the timing only)"}
    if not args.no_fp64_sample and ws == 1:
        # plain FP64 GPU path, one blob at a time (the reference's order): a stratified sample of the
        # blobs sorted by size, scaled to the whole ensemble
        order = sorted(range(args.blobs), key=lambda b: cells[b])
        pick = order[len(order) // 16::len(order) // 8][:8] if len(order) >= 8 else order
        tsum = 0.0
        for b in pick:
            f = lib.Blob(meshes[b], precision="fp64", **PHYS)
            f.update(1)
            tsum += f.update_timed(2, FLUSH_BYTES)["ms"] / 2
            f.close()
        est = tsum * len(order) / len(pick)
        out["fp64_path_sampled"] = {"value": sz["nodes"] / (est / 1e3), "ms_per_step_est": est,
                                    "sample_blobs": len(pick), "method": "FP64 single-blob path, blob by blob, "
                                    "stratified sample scaled to all blobs"}
        out["speedup_vs_fp64_path"] = out["value"] / out["fp64_path_sampled"]["value"]
    if not args.no_e2e and ws == 1:
        # end to end through the C ABI: every blob's host positions (pinned host memory) in, one step, every
        # blob's positions out
        pos, mem_kind = host_array((sum(m.n_nodes for m in meshes), 3))
        bt.positions(out=pos)
        ke = max(2, k // 4)
        t0 = time.perf_counter()
        for _ in range(ke):
            bt.set_positions(pos)
            bt.update(1)
            bt.positions(out=pos)
        e2e_s = time.perf_counter() - t0
        nb = 24 * sum(m.n_nodes for m in meshes)
        out["e2e"] = {"value": ws * sz["nodes"] * ke / e2e_s, "unit": "node-steps/s", "h2d_bytes_per_step": nb,
                      "d2h_bytes_per_step": nb, "steps": ke, "host_memory": mem_kind}
    bt.close()
    return out


def run_batch_long(args) -> dict:
    """The replica ensemble over a long run at a stable time step (the stiffest blobs are explicitly unstable at
    1e-12 s): per-blob equipartition of the strain energy at kT > 0, mean over samples after a burn-in of a fifth
    of the run, against (3 N_b - 6) kT / 2 (N_b vertices; the blobs carry no pins); and, at kT = 0 from a 2 %
    shear, the drift of a size-stratified sample of blobs from the FP64 single-blob path over the same steps.
    The explicit step of the overdamped dynamics holds each internal mode of rate lambda (V^-1 K) at
    1 / (1 - lambda dt / 2) of its kT / 2, so the ratio exceeds 1 where lambda dt is not small; the same sample
    of blobs is therefore also run through the FP64 single-blob path (the reference's arithmetic) from the same
    stream state, whose ratio the batch's must reproduce."""
    import numpy as np

    from ffea_ci_demo_gb300 import build, lib
    from ffea_ci_demo_gb300.mesh import apply_shear, ensemble

    build.build()
    meshes = ensemble(args.blobs)
    steps, dt, every = args.ensemble_long_steps, args.ensemble_long_dt, 10
    burn = steps // 5
    kw = {k: v for k, v in PHYS.items() if k != "solver"}
    kw["dt"] = dt
    bt = lib.Batch(meshes, **kw)
    order = sorted(range(len(meshes)), key=lambda b: meshes[b].n_elem)
    pick = sorted(set([order[0], order[len(order) // 3], order[2 * len(order) // 3], order[-1]]))
    rng0 = {b: bt.rng_state(b) for b in pick}
    t0 = time.perf_counter()
    samples = []
    for k in range(0, steps, every):
        bt.update(every)
        if k + every > burn:
            samples.append(bt.strain_energies())
    run_s = time.perf_counter() - t0
    bt.close()
    se = np.array(samples)
    kt_meso = PHYS["kT"] / (MESO_FORCE * MESO_LENGTH)
    nv = np.array([m.n_linear for m in meshes])
    want = kt_meso * (3 * nv - 6) / 2
    ratio = se.mean(axis=0) / want
    # one sample's relative spread is sqrt(2 / dof); the run's samples are correlated, so the per-blob z uses
    # the spread of its own sample means over four quarters of the sampled run
    q = np.array_split(se, 4, axis=0)
    qm = np.array([x.mean(axis=0) for x in q]) / want
    sem = qm.std(axis=0, ddof=1) / 2.0
    out = {"blobs": len(meshes), "steps": steps, "dt": dt, "burn_in_steps": burn, "sample_every": every,
           "samples": int(se.shape[0]), "run_s": run_s,
           "equipartition": {"ensemble_ratio": float(se.mean(axis=0).sum() / want.sum()),
                             "per_blob_ratio_mean": float(ratio.mean()), "per_blob_ratio_min": float(ratio.min()),
                             "per_blob_ratio_max": float(ratio.max()),
                             "per_blob_abs_dev_median": float(np.median(np.abs(ratio - 1))),
                             "blobs_within_5pct": int((np.abs(ratio - 1) < 0.05).sum()),
                             "per_blob_sem_median": float(np.median(sem))}}
    same = {}
    for b in pick:
        f = lib.Blob(meshes[b], precision="fp64", rng_state=rng0[b], **dict(PHYS, **kw))
        fs = []
        for k in range(0, steps, every):
            f.update(every)
            if k + every > burn:
                fs.append(f.measurements()["strain_energy"])
        f.close()
        same[str(b)] = {"tets": meshes[b].n_elem, "ratio_batch": float(ratio[b]),
                        "ratio_fp64_single_blob": float(np.mean(fs) / want[b])}
    out["equipartition"]["fp64_same_stream"] = same
    # the time-step bias on the smallest blob: the same simulated time at smaller steps (mixed single-blob path)
    b = pick[0]
    scan = []
    for div in (1, 2.5, 5, 10):
        dts = dt / div
        n_st = int(round(steps * div))
        f = lib.Blob(meshes[b], precision="mixed", rng_state=rng0[b], **dict(PHYS, **dict(kw, dt=dts)))
        ev = max(every, int(round(every * div)))
        fs = []
        for k in range(0, n_st, ev):
            f.update(ev)
            if k + ev > n_st // 5:
                fs.append(f.measurements()["strain_energy"])
        f.close()
        scan.append({"dt": dts, "steps": n_st, "ratio": float(np.mean(fs) / want[b])})
    out["equipartition"]["dt_scan_smallest_blob"] = {"blob": b, "tets": meshes[b].n_elem, "runs": scan}
    # kT = 0 drift against the FP64 single-blob path
    kw0 = dict(kw, kT=0.0, calc_noise=0)
    bt = lib.Batch(meshes, **kw0)
    x0 = [apply_shear(m, 0.02, seed=3) * (m.scale / MESO_LENGTH) for m in meshes]
    bt.set_positions(np.concatenate(x0))
    bt.update(steps)
    drift = {}
    for b in pick:
        f = lib.Blob(meshes[b], precision="fp64", **dict(PHYS, **kw0))
        f.set_state(pos=x0[b])
        f.update(steps)
        ref = f.pos()
        drift[str(b)] = {"tets": meshes[b].n_elem,
                         "max_abs_err_rel_to_max_disp": float(np.abs(bt.pos(b) - ref).max() /
                                                              np.abs(ref - x0[b]).max())}
        f.close()
    bt.close()
    out["kT0_drift_vs_fp64"] = drift
    return out


def run_adjoint(args) -> dict:
    """Configuration 3: gradient of a 200-step window (checkpoints every 20) of a 20^3-cell cube with
    lognormal per-element moduli, noise frozen (replayed), loss |x_K - target|^2; cost against the
    forward window."""
    import numpy as np

    from ffea_ci_demo_gb300 import build, lib
    from ffea_ci_demo_gb300.mesh import kuhn_cube

    build.build()
    n, steps, every = 20, args.adjoint_steps, 20
    mesh = kuhn_cube(n, side=5.0 * n, seed=12345)
    rng = np.random.default_rng(2025)
    mesh.material[:, 3] = rng.lognormal(np.log(5e8), 0.3, mesh.n_elem)
    mesh.material[:, 4] = rng.lognormal(np.log(5e8), 0.3, mesh.n_elem)
    s = mesh.scale / MESO_LENGTH
    target = mesh.pos * s + rng.normal(0.0, 0.01, size=mesh.pos.shape)
    out = {"workload": f"kuhn-cube-{n}: {mesh.n_elem} tets, {(n + 1) ** 3} nodes, G and K lognormal(ln 5e8, 0.3), "
                       f"NoMassCG, dt=1e-12 s, kT=4.11e-21 J (noise replayed), {steps}-step window, checkpoint every "
                       f"{every}, loss |x_K - target|^2", "steps": steps, "checkpoint_every": every}
    for prec in ("mixed", "fp64"):
        blob = lib.Blob(mesh, precision=prec, **PHYS)
        blob.update(2)
        adj = lib.Adjoint(blob, steps, every)
        t0 = time.perf_counter()
        adj.forward()
        t1 = time.perf_counter()
        d = blob.pos() - target
        g = adj.backward(2.0 * d)
        t2 = time.perf_counter()
        fwd, bwd = t1 - t0, t2 - t1
        out[prec] = {"forward_s": fwd, "backward_s": bwd, "grad_s_per_step": (fwd + bwd) / steps,
                     "gradient_cost_over_forward": (fwd + bwd) / fwd, "backward_over_forward": bwd / fwd,
                     "finite_gradients": bool(all(np.isfinite(g[k]).all() for k in ("G", "E", "A", "B")))}
        adj.close()
        blob.close()
    if args.adjoint_fd_steps > 0:
        out["fd_check"] = adjoint_fd_check(mesh, args.adjoint_fd_steps)
    return out


def adjoint_fd_check(mesh, steps: int) -> dict:
    """Central finite differences of the same loss on a shortened window at kT = 0 (8 sampled per-element
    parameters, relative step 1e-3, CG tolerance 1e-12 so that the solves' error stays below the differences'),
    evaluated with the FP64 GPU path (its trajectories follow the reference's to CG rounding), against the FP64
    and the mixed adjoint; relative error as a vector norm."""
    import copy

    import numpy as np

    from ffea_ci_demo_gb300 import lib
    from ffea_ci_demo_gb300.mesh import apply_shear

    kw = dict(PHYS, kT=0.0, calc_noise=0, epsilon=1e-12)
    rng = np.random.default_rng(7)
    x0 = apply_shear(mesh, 0.02, seed=3) * (mesh.scale / MESO_LENGTH)
    target = x0 + rng.normal(0.0, 0.05, size=x0.shape)
    samples = [(3, 17), (3, 23456), (4, 401), (4, 40000), (1, 999), (1, 31000), (2, 5), (2, 47000)]
    names = {1: "shear_visc", 2: "bulk_visc", 3: "shear_mod", 4: "bulk_mod"}

    def loss(m):
        b = lib.Blob(m, precision="fp64", **kw)
        b.set_state(pos=x0)
        b.update(steps)
        d = b.pos() - target
        b.close()
        return float((d * d).sum())

    fd = []
    for c, e in samples:
        h = 1e-3 * mesh.material[e, c]
        vals = []
        for sgn in (1, -1):
            m = copy.deepcopy(mesh)
            m.material[e, c] += sgn * h
            vals.append(loss(m))
        fd.append((vals[0] - vals[1]) / (2 * h))
    fd = np.array(fd)
    res = {"window_steps": steps, "samples": len(samples), "relative_step": 1e-3, "cg_epsilon": 1e-12,
           "fd_through": "FP64 GPU path, central differences, kT = 0"}
    for prec in ("fp64", "mixed"):
        b = lib.Blob(mesh, precision=prec, **kw)
        b.set_state(pos=x0)
        adj = lib.Adjoint(b, steps, 5)
        adj.forward()
        g = lib.meso_to_si_gradients(adj.backward(2.0 * (b.pos() - target)))
        got = np.array([g[names[c]][e] for c, e in samples])
        res[f"rel_err_{prec}"] = float(np.linalg.norm(got - fd) / np.linalg.norm(fd))
        adj.close()
        b.close()
    res["rel_err"] = max(res["rel_err_fp64"], res["rel_err_mixed"])
    return res


def run_scale(args) -> dict:
    """Configuration 4: the 64^3-cell cube (1,572,864 tets, 274,625 nodes, side 320 nm), CG_nomass and
    mass-lumped, mixed precision against the plain FP64 path: node-steps/s, HBM GB/s of the CG, CG
    iterations per step, and the mixed path's kT = 0 position error against the FP64 path."""
    import numpy as np

    from ffea_ci_demo_gb300 import build, lib
    from ffea_ci_demo_gb300.mesh import apply_shear, counts, kuhn_cube

    build.build()
    n = args.scale_cells
    mesh = kuhn_cube(n, side=5.0 * n, seed=12345)
    c = counts(n)
    N = c["N"]
    peak, peak_kind = measured_peak()
    out = {"workload": f"kuhn-cube-{n}: {c['T']} tets, {N} nodes, side {5 * n} nm, kT=4.11e-21 J",
           "cells_per_side": n, "tets": c["T"], "nodes": N}
    solvers = args.scale_solvers.split(",")
    precisions = args.scale_precisions.split(",")
    for solver, dt in (("CG_nomass", 1e-12), ("masslumped", args.scale_lumped_dt)):
        if solver not in solvers:
            continue
        res = {"dt": dt}
        for prec in precisions:
            b = lib.Blob(mesh, precision=prec, **dict(PHYS, solver=solver, dt=dt))
            b.update(2)
            deg = b.cg_preconditioner()[0]
            it0 = b.cg_iterations()[1]
            k = args.scale_steps
            t = b.update_timed(k, FLUSH_BYTES)
            it = (b.cg_iterations()[1] - it0) / k
            r = {"value": N * k / (t["ms"] / 1e3), "ms_per_step": t["ms"] / k, "cg_iters_per_step": it,
                 "phase_ms_per_step": {q: v / k for q, v in t["phase_ms"].items()}, "cg_kernel": b.cg_kernel()}
            if solver == "masslumped":
                # the value without the phase events (each costs a few microseconds inside a step of about a
                # tenth of a millisecond): the steps as update() runs them, timed around each graph launch
                kp = max(k, 50)
                tp = b.update_timed(kp, FLUSH_BYTES, phases=False)
                t = {"ms": tp["ms"] * k / kp, "phase_ms": t["phase_ms"]}
                r.update({"value": N * kp / (tp["ms"] / 1e3), "ms_per_step": tp["ms"] / kp,
                          "phase_events_ms_per_step": r["ms_per_step"]})
            p = 4 if prec == "mixed" else 8
            if solver == "CG_nomass":
                # the HBM anchor: at this size the matrix (165 MB mixed in SELL form) no longer fits in L2. The
                # bytes the format must stream per iteration (40 B per 3x3 block mixed, 76 B FP64, plus eight
                # vector passes) give the fraction; the per-unit model counts a scalar CSR (8 or 12 B per scalar
                # nonzero) and is reported as an equivalent rate only
                cg_ms = t["phase_ms"]["cg"] / k
                passes = it * (1 + deg)
                fmt = passes * cg_format_bytes_per_iteration(b.sizes()[2], N, p)
                model = passes * cg_bytes_per_iteration(n, p)
                name = f"{b.cg_kernel()}_{prec}_cube{n}"
                traffic = profiled(name, "dram_bytes_per_launch")
                r["roofline_cg"] = {
                    "bound": "hbm", "kernel": b.cg_kernel(), "achieved": fmt / (cg_ms / 1e3) / 1e9, "peak": peak,
                    "unit": "GB/s", "frac": fmt / (cg_ms / 1e3) / 1e9 / peak, "peak_source": peak_kind,
                    "bytes": "SELL format per iteration x iterations", "ms_per_launch": cg_ms,
                    "traffic": traffic, "traffic_source": f"profiles/{name}.txt" if traffic else None,
                    "dram_frac": (traffic / (cg_ms / 1e3) / 1e9 / peak) if traffic else None,
                    "model_equiv_gbs": model / (cg_ms / 1e3) / 1e9,
                    "preconditioner": f"chebyshev degree {deg}" if deg else "jacobi"}
            else:
                step_bytes = masslumped_bytes_per_step(n, p)
                el_ms = t["phase_ms"]["element"] / k
                ek = "element_mixed_kernel" if prec == "mixed" else "element_kernel"
                prof = f"{ek}_lumped_cube{n}" if prec == "mixed" else f"element_kernel_{prec}_lumped_cube{n}"
                r["roofline"] = {"bound": "hbm", "kernel": f"whole step ({ek} dominant)",
                                 "achieved": step_bytes / (t["ms"] / k / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                                 "frac": step_bytes / (t["ms"] / k / 1e3) / 1e9 / peak, "peak_source": peak_kind,
                                 "bytes_per_step": step_bytes, "element_ms_per_step": el_ms,
                                 "traffic_element": profiled(prof, "dram_bytes_per_launch")}
            res[prec] = r
            b.close()
        if "mixed" in res and "fp64" in res:
            res["speedup_mixed_vs_fp64"] = res["mixed"]["value"] / res["fp64"]["value"]
        # kT = 0 error of the mixed path against the FP64 path (same initial shear)
        if args.scale_error_steps > 0:
            p0 = apply_shear(mesh, 0.02, seed=3) * (mesh.scale / MESO_LENGTH)
            xs = {}
            for prec in ("fp64", "mixed"):
                b = lib.Blob(mesh, precision=prec, **dict(PHYS, solver=solver, dt=dt, kT=0.0, calc_noise=0))
                b.set_state(pos=p0)
                b.update(args.scale_error_steps)
                xs[prec] = b.pos()
                b.close()
            res["kT0_error"] = {"steps": args.scale_error_steps,
                                "max_abs_disp_err_rel_to_max_disp":
                                    float(np.abs(xs["mixed"] - xs["fp64"]).max() / np.abs(xs["fp64"] - p0).max())}
        out[solver] = res
    return out


CPU_FLAGS = "-O3 -ffast-math -fopenmp (the reference's release flags without -march=native: the same build " \
            "must give the same results on x86 and Arm hosts)"


def cpu_sample(n: int, threads: int, budget_s: float, max_steps: int, warmup: int = 1):
    """Time the oracle (reference algorithm, release optimisation, OpenMP) on the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    from ffea_ci_demo_gb300.mesh import counts, kuhn_cube

    pyoracle.build()
    mesh = kuhn_cube(n, side=SIDE * n / N_CELLS, seed=12345)
    o = pyoracle.OracleBlob(mesh, threads=threads, fast=True, **PHYS)
    for _ in range(warmup):
        o.step(1)
    done, t0 = 0, time.perf_counter()
    while done < max_steps:
        if o.step(1) != 0:
            break
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    N = counts(n)["N"]
    return {"value": N * done / dt, "unit": "node-steps/s", "cores": threads, "kind": "port",
            "sample": f"{done} full steps (after {warmup} warm-up) of the {n}^3-cell cube, {N} nodes, "
                      f"{o.total_cg_iters() / max(1, done + warmup):.0f} CG iterations/step",
            "seconds": dt, "steps": done, "cpu_model": cpu_model(), "flags": CPU_FLAGS}


def headline_roofline(args, head: dict) -> dict:
    """Roofline of the headline CG launch. The unit is one CG iteration by the per-unit model,
    nnz (p + 4) + (R + 1) 4 + 8 R p bytes, so achieved = iterations x that / launch time (CUDA events on the
    blob's stream) against the measured HBM copy rate. The Chebyshev preconditioner's extra matrix passes are
    listed apart, at their own bytes (matrix + two vector passes). A matrix that stays in L2 is bounded by L2
    and synchronisation, not HBM: the `l2` object gives the L2 (lts) throughput and the DRAM bytes that ncu
    measured on one full-size launch (profiles/)."""
    peak, peak_kind = measured_peak()
    p = 4 if args.headline == "mixed" else 8
    iters = head["cg_iters_per_step"]
    deg = head["cg_poly"]
    cg_ms = head["phase_ms"]["cg"] / head["steps"]
    unit = cg_bytes_per_iteration(args.cells, p)
    achieved = iters * unit / (cg_ms / 1e3) / 1e9
    extra = iters * deg * cheb_pass_bytes(args.cells, p)
    kernel = head["cg_kernel"]
    prof = f"{kernel}_{args.headline}_cube{args.cells}"
    traffic = profiled(prof, "dram_bytes_per_launch")
    l2_resident = head["blocks"] * (9 * p + 4) <= 64e6
    r = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
         "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
         "unit_of_work": "one CG iteration (per-unit model bytes)", "bytes_per_unit": unit,
         "units_per_launch": iters, "ms_per_launch": cg_ms,
         "preconditioner": f"chebyshev degree {deg} (lambda_max {head['lambda_max']:.4f})" if deg else "jacobi"}
    if deg:
        r["chebyshev_passes"] = {"passes_per_launch": iters * deg, "bytes_per_pass": cheb_pass_bytes(args.cells, p),
                                 "achieved_incl_passes": (iters * unit + extra) / (cg_ms / 1e3) / 1e9}
    if l2_resident:
        lts = profiled(prof, "lts_throughput_pct")
        r["l2"] = {"bound": "l2", "matrix_bytes_sell": head["blocks"] * (9 * p + 4),
                   "lts_throughput_frac": lts / 100 if lts is not None else None,
                   "dram_bytes_per_launch": traffic, "source": f"profiles/{prof}.txt",
                   "note": "the matrix stays in L2 (and partly in shared memory) across the launch's matrix passes; "
                           "DRAM sees about one read of it per launch after the L2 flush, so the launch is bound by "
                           "L2 latency and grid synchronisation, and the HBM fraction is a rate, not HBM use"}
    return r


def summary(line: dict) -> dict:
    """The figures a reader needs first, repeated compactly at the end of the line."""
    def g(d, *ks):
        for k in ks:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d

    def r3(x):
        return None if x is None else float(f"{x:.4g}")

    out = {"value": r3(line.get("value")), "e2e": r3(g(line, "e2e", "value")),
           "ms_per_step": r3(line.get("ms_per_step")), "roofline_frac": r3(g(line, "roofline", "frac")),
           "l2_frac": r3(g(line, "roofline", "l2", "lts_throughput_frac")),
           "fp64_value": r3(g(line, "fp64_path", "value")), "mixed_over_fp64": r3(line.get("speedup_vs_fp64_path")),
           "kT0_err_1000": r3(g(line, "error", "max_abs_disp_err_rel_to_max_disp")),
           "kT0_err_steps": g(line, "error", "kT0_steps"),
           "batch_value": r3(g(line, "batched", "value")), "batch_e2e": r3(g(line, "batched", "e2e", "value")),
           "batch_frac_format": r3(g(line, "batched", "roofline", "frac")),
           "batch_over_fp64": r3(g(line, "batched", "speedup_vs_fp64_path")),
           "scale_nomass_mixed": r3(g(line, "scale", "CG_nomass", "mixed", "value")),
           "scale_nomass_frac": r3(g(line, "scale", "CG_nomass", "mixed", "roofline_cg", "frac")),
           "scale_lumped_mixed": r3(g(line, "scale", "masslumped", "mixed", "value")),
           "scale_lumped_frac": r3(g(line, "scale", "masslumped", "mixed", "roofline", "frac")),
           "adjoint_cost_mixed": r3(g(line, "adjoint", "mixed", "gradient_cost_over_forward")),
           "adjoint_fd_rel_err": r3(g(line, "adjoint", "fd_check", "rel_err")),
           "cpu": r3(g(line, "cpu_baseline", "value")), "cpu_1thread": r3(g(line, "cpu_baseline", "value_1_thread"))}
    return {k: v for k, v in out.items() if v is not None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["both", "mixed", "fp64"], default="both")
    ap.add_argument("--cells", type=int, default=N_CELLS)
    ap.add_argument("--error-steps", type=int, default=1000,
                    help="kT = 0 steps of the mixed against the FP64 path (the stated bound is for 1000)")
    ap.add_argument("--kt-steps", type=int, default=200, help="kT > 0 comparison of the two paths (0: skip)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cpu-1thread", action="store_true", help="skip the 1-thread CPU step")
    ap.add_argument("--workload", choices=["both", "single", "batch", "scale"], default="both",
                    help="single: the 40^3 blob (headline); batch: the replica ensemble; scale: the 64^3 cube only "
                         "(a JSON object, not a bench line; for profiling); both: all in one line")
    ap.add_argument("--blobs", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=10,
                    help="timed steps of the replica ensemble (its stiffest blobs are explicitly unstable at "
                         "dt = 1e-12 s: they invert an element after about 20 steps, in the reference's algorithm "
                         "too, so warm-up + timed steps stay below that)")
    ap.add_argument("--ensemble-long-steps", type=int, default=0,
                    help="batch: also run the ensemble this many steps at --ensemble-long-dt for the per-blob "
                         "equipartition and the kT=0 drift against FP64 (0: skip; 1000 takes about four minutes)")
    ap.add_argument("--ensemble-long-dt", type=float, default=5e-13)
    ap.add_argument("--no-tune", action="store_true", help="batch: fixed launch configuration (--cg-threads, --tpn)")
    ap.add_argument("--cg-threads", type=int, default=128)
    ap.add_argument("--tpn", type=int, default=1)
    ap.add_argument("--no-fp64-sample", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--adjoint-steps", type=int, default=200)
    ap.add_argument("--adjoint-fd-steps", type=int, default=20,
                    help="window of the adjoint's finite-difference check (0: skip)")
    ap.add_argument("--no-scale", action="store_true")
    ap.add_argument("--scale-cells", type=int, default=64)
    ap.add_argument("--scale-steps", type=int, default=5)
    ap.add_argument("--scale-error-steps", type=int, default=20)
    ap.add_argument("--scale-lumped-dt", type=float, default=1e-12)
    ap.add_argument("--scale-solvers", default="CG_nomass,masslumped")
    ap.add_argument("--scale-precisions", default="mixed,fp64")
    ap.add_argument("--no-adjoint", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    args.headline = "fp64" if args.precision == "fp64" else "mixed"
    ws, rank, local = rank_info()
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        # each step is one full blob step of the same workload, run by the reference algorithm on all host
        # cores; the number of timed steps is capped so that the run stays within a few minutes
        r = cpu_sample(args.cells, threads, budget_s=150.0, max_steps=args.steps, warmup=args.warmup)
        line = {"metric": "node-steps/s", "value": r["value"], "unit": "node-steps/s", "n_gpus": args.gpus,
                "steps": r["steps"], "warmup": args.warmup, "ms_per_step": 1e3 * r["seconds"] / r["steps"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded Kuhn cube)", "config": workload_config(args.cells, "fp64"),
                "impl": "reference",
                "cpu_baseline": {k: r[k] for k in ("value", "unit", "cores", "kind", "sample", "cpu_model", "flags")},
                "e2e": {"value": r["value"], "unit": "node-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    pick_device(local)
    if args.workload == "scale":
        if rank == 0:
            print(json.dumps({"scale": run_scale(args)}), flush=True)
        return
    if args.workload == "batch":
        args.steps = args.batch_steps
        ranks = Replicas(ws) if ws > 1 else None
        b = run_batch(args, ws, rank, ranks)
        if ranks:
            ranks.close()
        if rank != 0:
            return
        if args.ensemble_long_steps > 0 and ws == 1:
            b["long_run"] = run_batch_long(args)
        line = {"metric": "node-steps/s", "value": b["value"], "unit": "node-steps/s", "n_gpus": ws,
                "steps": b["steps"], "warmup": args.warmup, "ms_per_step": b["ms_per_step"],
                "higher_is_better": True, "scaling": "strong" if ws > 1 else "weak", "vs_baseline": None,
                "dtype": "f32+f64", "data": "synthetic (seeded Kuhn-cube ensemble)",
                "config": {"workload": b["workload"], "blobs": b["blobs"], "nodes": b["nodes"], "tets": b["tets"],
                           "l2": "flushed before every timed step (256 MiB scratch write)",
                           "parallelism": f"ensemble sharded x{ws}" if ws > 1 else "replicas x1"},
                "clocks": b["clocks"], "e2e": b.get("e2e"), "gpu_launches": b["gpu_launches"],
                "roofline": b["roofline"], "batched": b}
        print(json.dumps(line), flush=True)
        return
    res = run_gpu_arm(args, ws, rank, local)
    if rank != 0:
        return
    head = res[args.headline]
    line_roofline = headline_roofline(args, head)
    line = {"metric": "node-steps/s", "value": head["value"], "unit": "node-steps/s", "n_gpus": ws,
            "steps": head["steps"], "warmup": args.warmup, "ms_per_step": head["ms"] / head["steps"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if args.headline == "mixed" else "f64", "data": "synthetic (seeded Kuhn cube)",
            "config": dict(workload_config(args.cells, args.headline), parallelism=f"replicas x{ws}"),
            "clocks": head["clocks"], "e2e": head["e2e"], "gpu_launches": head["launches"],
            "roofline": line_roofline,
            "phase_ms_per_step": {k: v / head["steps"] for k, v in head["phase_ms"].items()},
            "cg_iters_per_step": head["cg_iters_per_step"]}
    if "fp64" in res and args.headline != "fp64":
        f = res["fp64"]
        line["fp64_path"] = {"value": f["value"], "ms_per_step": f["ms"] / f["steps"], "steps": f["steps"],
                             "cg_iters_per_step": f["cg_iters_per_step"], "preconditioner": "jacobi",
                             "phase_ms_per_step": {k: v / f["steps"] for k, v in f["phase_ms"].items()}}
        line["speedup_vs_fp64_path"] = head["value"] / f["value"]
    if "error" in res:
        line["error"] = res["error"]
    if args.workload == "both" and ws == 1:
        k = args.steps
        args.steps = args.batch_steps
        line["batched"] = run_batch(args, ws)
        args.steps = k
        if not args.no_adjoint:
            line["adjoint"] = run_adjoint(args)
        if not args.no_scale:
            line["scale"] = run_scale(args)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sample(args.cells, os.cpu_count() or 1, budget_s=20.0, max_steps=3)
        line["cpu_baseline"].pop("seconds")
        line["cpu_baseline"].pop("steps")
        if not args.no_cpu_1thread:
            one = cpu_sample(args.cells, 1, budget_s=0.0, max_steps=1, warmup=0)
            line["cpu_baseline"]["value_1_thread"] = one["value"]
            line["cpu_baseline"]["sample_1_thread"] = one["sample"]
    line["summary"] = summary(line)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
