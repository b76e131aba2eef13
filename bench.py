"""Benchmark: matrix-free XXZ H*v on the L=1000, N_down=4 chain sector (k=0).

Workload (one "step" = one complex(8) H*v over the whole sector, D ~ 4.1e7
representatives): periodic XXZ chain L=1000, nearest-neighbour Jxy=1, Jz=0.5,
next-nearest J2xy=J2z=0.3, h=0, sector N_down=4, k=0.  Synthetic: the bond
list is generated, x is a seeded random vector.

metric  = algorithmic HBM bytes of one H*v / time, with
          B = D*(16 [x_i] + 16 [y_i] + 8 [list_s_i] + 8 [list_r_i])
            + nnz_off*(16 [x_id] + 8 [list_r_id])
          nnz_off = exact number of off-diagonal (row, col) entries.
value   = B / device time per step (inputs resident in HBM, x and y 663 MB
          each, larger than L2), CUDA events on the launching stream.
e2e     = the same B / wall time of qs3g_hv called with HOST buffers
          (pinned), i.e. H2D of x + kernel + D2H of y every step.

--impl reference times the CPU restatement of ham_to_vec_wave_vector (the
reference has no GPU path and cannot index this sector with its 32-bit
integers) on the host cores over a bounded sample of rows, extrapolated to a
full H*v.  N>1 GPUs run independent replicas (the path needs no exchange on
one sector; multi-GPU sharding is not built).
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L_SITES, NOD = 1000, 4
J1, J2 = (1.0, 0.5), (0.3, 0.3)
WORKLOAD = "xxz_chain_L1000_Ndown4_k0_J1(1,0.5)_J2(0.3,0.3)_complex128_hv"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def peaks_bf16():
    """Measured dense BF16 tensor rate (burst), TFLOP/s; the fallback figure otherwise."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f).get("bf16_tflops", 1900.0))
    return 1900.0


def traffic_record():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons, one streaming process sampling every 100 ms
    while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._p = None
        self._t = None

    def _reader(self):
        for line in self._p.stdout:
            line = line.strip()
            if line:
                self.samples.append([s.strip() for s in line.split(",")])

    def __enter__(self):
        try:
            self._p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                        "--format=csv,noheader,nounits", "-lms", "100"],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._reader, daemon=True)
            self._t.start()
            t0 = time.time()
            while not self.samples and time.time() - t0 < 3.0:
                time.sleep(0.02)
        except Exception:
            self._p = None
        return self

    def __exit__(self, *a):
        if self._p is not None:
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()
            self._t.join(timeout=5)

    def summary(self):
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            for k, n in enumerate(names):
                if len(s) > 3 + k and s[3 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch.distributed as dist
    backend = os.environ.get("QS3G_BENCH_BACKEND", "nccl")
    dist.init_process_group(backend=backend)
    return dist.get_rank(), dist.get_world_size(), int(os.environ.get("LOCAL_RANK", "0")), dist


def max_over_ranks(v: float, dist, device=None) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist, device=None):
    if dist is not None:
        if device is not None:
            dist.barrier(device_ids=[device.index]) if device.type == "cuda" else dist.barrier()
        else:
            dist.barrier()


def chain_lists_cpu(nthreads):
    """Sector lists for the workload, enumerated on the CPU (anchored candidates)."""
    from oracle import oracle as O
    return O.chain_sector_lists(L_SITES, NOD, 0, nthreads)


def workload_config(D, world):
    """The workload as both arms name it (the reference arm and the GPU arm print the same dict)."""
    return {"workload": WORKLOAD, "sector_dim": int(D), "parallelism": f"replicas{world}",
            "l2": "inputs larger than L2 (x, y 16*D bytes each), no flush"}


def run_reference(args, rank, world, dist):
    from oracle import oracle as O
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    ls, lr = chain_lists_cpu(nthreads)
    D = len(ls)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(D) + 1j * rng.standard_normal(D)
    from ed_gb300 import inputs
    bonds, jxy, jz = inputs.chain_bonds(L_SITES, J1, J2)
    m = O.Model(L_SITES, L_SITES, 1, 1, bonds, jxy, jz, kmax=NOD + 2)
    sec = O.Sector(m, NOD, (0, 0, 0), ls, lr)
    # calibrate a sample of about args.cpu_seconds / (steps + warmup) per step
    r0 = D // 3
    t0 = time.perf_counter()
    sec.hv(x, rows=(r0, r0 + 2000), nthreads=nthreads)
    per_row = (time.perf_counter() - t0) / 2000
    rows = int(max(2000, min(D - r0, args.cpu_seconds / max(1, args.steps + args.warmup) / per_row)))
    nnz_rows = O.count_offdiag_rows(sec, r0, r0 + rows, nthreads)
    Bs = rows * 48 + nnz_rows * 24
    for _ in range(args.warmup):
        sec.hv(x, rows=(r0, r0 + rows), nthreads=nthreads)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        sec.hv(x, rows=(r0, r0 + rows), nthreads=nthreads)
        ts.append(time.perf_counter() - t0)
    t = float(np.mean(ts))
    value = Bs / t / 1e9
    sample = f"{rows} rows of {D} (rows {r0}..{r0 + rows - 1}), extrapolated per byte to a full H*v"
    line = {
        "impl": "reference", "metric": "hv_algorithmic_hbm_gbs", "value": value, "unit": "GB/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(D, world),
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": nthreads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args, rank, world, local_rank, dist):
    import torch
    from ed_gb300 import capi, inputs
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    bonds, jxy, jz = inputs.chain_bonds(L_SITES, J1, J2)
    h = capi.Handle(L_SITES, L_SITES, 1, 1, bonds, jxy, jz)
    stream = torch.cuda.current_stream(dev)
    h.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    D = h.build_sector(NOD, (0, 0, 0))
    torch.cuda.synchronize(dev)
    t_build = time.perf_counter() - t0
    nnz = int(h.connection_table_count())
    B = D * 48 + nnz * 24
    g = torch.Generator(device="cpu").manual_seed(1234 + rank)
    xr = torch.randn(D, 2, dtype=torch.float64, generator=g)
    x = torch.view_as_complex(xr).to(dev)
    y = torch.empty_like(x)
    # warm-up
    for _ in range(args.warmup):
        h.hv_device(x.data_ptr(), y.data_ptr())
    torch.cuda.synchronize(dev)
    # timed region: inputs (663 MB each) exceed the 129 MB L2, no flush needed
    n0 = capi.kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(dist, dev)
    torch.cuda.synchronize(dev)
    with ClockSampler(local_rank) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            h.hv_device(x.data_ptr(), y.data_ptr())
        ev1.record(stream)
        torch.cuda.synchronize(dev)
    barrier(dist, dev)
    launches = capi.kernel_launches() - n0
    ms = ev0.elapsed_time(ev1) / args.steps
    ms = max_over_ranks(ms, dist, dev)
    value = world * B / (ms * 1e-3) / 1e9
    # e2e: host buffers through the C ABI (H2D x + H*v + D2H y every step)
    xh = torch.empty(D, dtype=torch.complex128, pin_memory=True)
    xh.copy_(x.cpu())
    yh = torch.empty(D, dtype=torch.complex128, pin_memory=True)
    xnp, ynp = xh.numpy(), yh.numpy()
    h.hv_host_into(xnp, ynp)
    e2e_steps = max(1, min(args.steps, 5))
    barrier(dist, dev)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        h.hv_host_into(xnp, ynp)
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    t_e2e = max_over_ranks(t_e2e, dist, dev)
    # check the e2e result against the device result (same x)
    yd = y.cpu().numpy()
    assert np.abs(ynp - yd).max() <= 1e-12 * np.abs(yd).max()
    peak, peak_kind = peaks()
    achieved = B / (ms * 1e-3) / 1e9
    tr = traffic_record().get("hv_chain64", {})
    line = {
        "metric": "hv_algorithmic_hbm_gbs", "value": value, "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(D, world),
        "hv_bytes": {"nnz_offdiag": nnz, "bytes_per_hv": B, "per_row": 48, "per_offdiag_entry": 24},
        "sector_build_s": t_build,
        "hv_per_s": world * 1e3 / ms,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": tr.get("dram_bytes_per_launch"),
                     "traffic_source": tr.get("source")},
        "e2e": {"value": world * B / t_e2e / 1e9, "unit": "GB/s", "h2d_bytes_per_step": 16 * D,
                "d2h_bytes_per_step": 16 * D, "ms_per_step": t_e2e * 1e3},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    line["hv_variants"] = hv_variants(h, x, D, stream, dev)
    # the product the ground-state solve runs: real FP32 from the cached
    # connection table, against HBM with the bytes it streams
    tv = line["hv_variants"].get("table_real_f32")
    if tv:
        trt = traffic_record().get("hv_tab_real_f32", {})
        line["roofline_table_real_f32"] = {
            "bound": "hbm", "achieved": tv["stream_gbs"], "peak": peak, "unit": "GB/s",
            "frac": tv["stream_gbs"] / peak, "peak_kind": peak_kind, "ms": tv["ms"],
            "streamed_bytes": line["hv_variants"]["table"]["bytes"] + D * (2 * 4 + 16),
            "traffic": trt.get("dram_bytes_per_launch"), "traffic_source": trt.get("source")}
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"], line["parity"] = cpu_leg(args, h, x, y, D)
    h.close()
    if args.solve and rank == 0 and world == 1:
        line["gs_solve"] = solve_bench(args)
    if args.dsf and rank == 0:
        line["dsf_batch"] = dsf_bench()
    if args.batch and world == 1:
        line["batched_solves"] = batch_bench(args)
    if args.cfg5 and rank == 0 and world == 1:
        line["cfg5_learned_start"] = cfg5_bench(args)
    if rank == 0:
        print(json.dumps(line), flush=True)


def hv_variants(h, x, D, stream, dev, reps=10):
    """CUDA-event time of the other forms of the same product on the same sector
    (real vectors: k = 0, H real symmetric): real FP64, complex(4) and real
    FP32, each with its algorithmic bytes D*(2 s + 16) + nnz_off*(s + 8)."""
    import torch
    from ed_gb300 import capi
    nnz = int(h.connection_table_count())
    out = {}
    xr = x.real.contiguous()
    x32 = x.to(torch.complex64)
    xr32 = xr.to(torch.float32)
    forms = [("real_f64", lambda a, b: h.hv_real_device(a, b), xr, 8),
             ("complex_f32", lambda a, b: h.hv32_device(a, b), x32, 8),
             ("real_f32", lambda a, b: h.hv32_real_device(a, b), xr32, 4)]
    def timed(fn, xv):
        yv = torch.empty_like(xv)
        for _ in range(3):
            fn(xv.data_ptr(), yv.data_ptr())
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        ev0.record(stream)
        for _ in range(reps):
            fn(xv.data_ptr(), yv.data_ptr())
        ev1.record(stream)
        torch.cuda.synchronize(dev)
        return ev0.elapsed_time(ev1) / reps, yv

    for name, fn, xv, s in forms:
        ms, yv = timed(fn, xv)
        B = D * (2 * s + 16) + nnz * (s + 8)
        out[name] = {"ms": ms, "algorithmic_gbs": B / (ms * 1e-3) / 1e9}
        del yv
    # the same products from the cached connection table (qs3g_hv_cache):
    # stream_gbs counts what the table form streams from HBM (table, x, y,
    # diagonal, configuration: nb + D * (2 s + 16)); gathers of x(id) hit L2
    _, y_mf = timed(lambda a, b: h.hv_device(a, b), x)
    t0 = time.perf_counter()
    nb = h.hv_cache(True)
    torch.cuda.synchronize(dev)
    tb = time.perf_counter() - t0
    out["table"] = {"bytes": nb, "build_s": tb}
    for name, fn, xv, s in [("complex_f64", lambda a, b: h.hv_device(a, b), x, 16)] + forms:
        ms, yv = timed(fn, xv)
        B = D * (2 * s + 16) + nnz * (s + 8)
        out["table_" + name] = {"ms": ms, "algorithmic_gbs": B / (ms * 1e-3) / 1e9,
                                "stream_gbs": (nb + D * (2 * s + 16)) / (ms * 1e-3) / 1e9}
        if name == "complex_f64":
            out["table_complex_f64"]["bit_identical_to_matrix_free"] = bool(torch.equal(yv, y_mf))
        del yv
    # complex(8) from the table in double-float arithmetic (qs3g_hv_df)
    ms, yv = timed(lambda a, b: h.hv_df_device(a, b), x)
    B = D * 48 + nnz * 24
    out["table_complex_f64_df"] = {
        "ms": ms, "algorithmic_gbs": B / (ms * 1e-3) / 1e9, "stream_gbs": (nb + D * 48) / (ms * 1e-3) / 1e9,
        "max_rel_dev_from_fp64": float((yv - y_mf).abs().max() / y_mf.abs().max())}
    del yv
    h.hv_cache(False)
    return out


def cpu_leg(args, h, x, y, D):
    """The oracle on this host's cores: (1) timed on a bounded sample of rows
    (cpu_baseline, extrapolated per byte); (2) the parity of the timed GPU
    product on the same rows -- the oracle's own enumeration of the sector
    (list_s bit for bit, list_r), its ham_to_vec_wave_vector on the sampled
    rows against the GPU y of the timed region (same x), and the connection
    table of 2,000 rows bit for bit."""
    from oracle import oracle as O
    from ed_gb300 import inputs
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ls, lr = O.chain_sector_lists(L_SITES, NOD, 0, nthreads)
    t_lists = time.perf_counter() - t0
    lsg, lrg = h.get_sector()
    bonds, jxy, jz = inputs.chain_bonds(L_SITES, J1, J2)
    om = O.Model(L_SITES, L_SITES, 1, 1, bonds, jxy, jz, kmax=NOD + 2)
    sec = O.Sector(om, NOD, (0, 0, 0), ls, lr)
    xc = x.cpu().numpy()
    r0 = D // 3
    t0 = time.perf_counter()
    sec.hv(xc, rows=(r0, r0 + 2000), nthreads=nthreads)
    per_row = (time.perf_counter() - t0) / 2000
    rows = int(max(2000, min(D - r0, args.cpu_seconds / per_row)))
    nnz_rows = O.count_offdiag_rows(sec, r0, r0 + rows, nthreads)
    t0 = time.perf_counter()
    yc = sec.hv(xc, rows=(r0, r0 + rows), nthreads=nthreads)[r0:r0 + rows]
    tc = time.perf_counter() - t0
    cpu = {"value": (rows * 48 + nnz_rows * 24) / tc / 1e9, "unit": "GB/s", "cores": nthreads,
           "kind": "port", "sample": f"{rows} rows of {D} timed (rows {r0}..{r0 + rows - 1}), "
                                     f"extrapolated per byte"}
    yg = y[r0:r0 + rows].cpu().numpy()
    err = float(np.abs(yg - yc).max() / np.abs(yc).max())
    # per-row tolerance: 1e-13 of max|y| plus the rounding bound of the reference's
    # diagonal, a running sum over all NOxxz bonds (ham2vec_v3.f90:56-67)
    tol = 1e-13 * np.abs(yc).max() + len(jz) * 2.0 ** -53 * np.abs(0.25 * jz).sum() * np.abs(xc[r0:r0 + rows])
    over = float((np.abs(yg - yc) / tol).max())
    c0, c1 = D // 5, D // 5 + 2000
    ro, co, eo, bo = sec.connection_table(nthreads, rows=(c0, c1))
    rg, cg, eg, bg = h.connection_table(rows=(c0, c1))
    table_equal = bool(np.array_equal(rg, ro + 1) and np.array_equal(cg, co + 1) and
                       np.array_equal(eg, eo) and np.array_equal(bg, bo + 1))
    parity = {"oracle": "CPU restatement of ham_to_vec_wave_vector / representative_SQ / findstate",
              "list_s_equal": bool(np.array_equal(lsg, ls)),
              "list_r_max_rel_err": float(np.abs(lrg / lr - 1.0).max()),
              "hv_rows": rows, "hv_max_rel_err": err,
              "hv_tol": "per row: 1e-13*max|y| + NOxxz*2^-53*sum|Jz/4|*|x_i| (the reference's diagonal sum)",
              "hv_max_err_over_tol": over,
              "table_rows": c1 - c0, "table_entries": int(len(ro)), "table_bit_exact": table_equal,
              "oracle_lists_s": t_lists}
    parity["ok"] = bool(parity["list_s_equal"] and parity["list_r_max_rel_err"] <= 1e-15 and
                        over <= 1.0 and table_equal)
    return cpu, parity


ARMS = {  # name: (qs3g_trlan precision, learned start)
    "learned_fp32_real": (1 | 8, True), "learned_fp32": (1, True), "random_fp32_real": (1 | 8, False),
    "random_fp32": (1, False), "random_fp64_real": (0 | 8, False), "random_df": (2, False),
    "plain_fp64_random": (0, False),
}


def solve_arm(args):
    """One arm of the ground-state solve alone (--arm NAME), stopped after
    --arm-limit seconds: for profiling the solver on the benchmark chain."""
    from ed_gb300 import capi, learned
    prec, use_net = ARMS[args.arm]
    delta, j2 = J1[1], J2[0]
    v = None
    h = learned.chain_handle(args.L, delta, j2)
    if use_net:
        net = capi.Mlp(seed=1)
        learned.generate(net, learned.training_problems(seed=1))
        learned.train(net, rounds=10, steps=300, batch=4096, lr=2e-3)
    D = h.build_sector(NOD, (0, 0, 0))
    if use_net:
        v = learned.start_vector(net, h, delta, j2)
    if args.table:
        h.hv_cache(True)
    h.set_time_limit(args.arm_limit)
    t0 = time.perf_counter()
    r = h.trlan(1, args.nok, args.nom, maxitr=args.maxrestart, tol=args.tol, precision=prec, conv_mode=1, seed=7,
                start=v, want_psi=False, allow_unconverged=True)
    dt = time.perf_counter() - t0
    st = h.trlan_stats()
    h.close()
    print(json.dumps({"arm": args.arm, "L": args.L, "sector_dim": D, "seconds": dt, "E0": float(r["ene"][0]),
                      "resid": float(r["resid"][0]), "converged": bool(r["converged"]), "hv": r["iters"],
                      "hv_fp32": st["hv_fp32"], "hv_fp64": st["hv_fp64"], "restarts": st["restarts"],
                      "timed_out": st["timed_out"]}), flush=True)


def mlp_inference_rate(net, h, D, delta, j2, reps=3):
    """Tensor-core rate of the network's inference over the sector: D
    representatives x NOD rotations, 2 (16*128 + 2*128*128 + 128) FLOP per
    evaluation over the time of a device-output prediction call.  The call
    returns when its work is done, so the events bracket it whole, including
    its host-side staging: a lower bound on the kernels' rate."""
    import torch
    from ed_gb300 import learned
    dev = torch.device("cuda", torch.cuda.current_device())
    vd = torch.empty(D, dtype=torch.complex128, device=dev)
    c = learned.cond(delta, j2)
    net.predict_device(h, *c, vd.data_ptr())
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        net.predict_device(h, *c, vd.data_ptr())
    e1.record()
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / reps
    evals = D * NOD
    flop = evals * 2 * (16 * 128 + 2 * 128 * 128 + 128)
    peak = peaks_bf16()
    tf = flop / (ms * 1e-3) / 1e12
    del vd
    return {"evaluations": evals, "ms": ms, "tflops": tf, "peak_bf16_tflops": peak,
            "frac": tf / peak if peak else None}


def solve_bench(args):
    """Ground state of the benchmark chain (L, N_down=4, k=0, Delta=0.5, J2=0.3,
    an unseen point of the network's training range) to ||H psi - E psi|| <= tol,
    the residual recomputed in FP64 from the returned vector:

      learned_fp32_real  the network's start vector (trained here on chains
                         L = 48..128 whose ground states the GPU TRLan computes
                         first), precision 1: every Krylov vector in FP32,
                         anchored on one FP64 vector, FP64-accurate reductions,
                         real vectors (k = 0: H is real symmetric);
      plain_fp64_random  the reference's arithmetic: complex(8) vectors, FP64
                         throughout, random start (eigen_solver.f90:92-96),
                         stopped at plain_limit seconds if it has not converged.
    --solve-all adds the same start and storage with complex vectors, complex(4)
    storage from a random start, FP64 real vectors from a random start and
    double-float arithmetic from a random start."""
    from ed_gb300 import capi, learned
    delta, j2 = J1[1], J2[0]
    out = {"workload": f"xxz_chain_L{args.L}_Ndown4_k0_Delta{delta}_J2_{j2}", "tol": args.tol,
           "NOK": args.nok, "NOM": args.nom, "conv": "FP64-recomputed residual <= tol"}
    t0 = time.perf_counter()
    net = capi.Mlp(seed=1)
    learned.generate(net, learned.training_problems(seed=1))
    t_gen = time.perf_counter() - t0
    learned.train(net, rounds=10, steps=300, batch=4096, lr=2e-3)
    out["network"] = {"generate_s": t_gen, "train_s": time.perf_counter() - t0 - t_gen,
                      "loss": float(net.loss_grad()[0])}
    h = learned.chain_handle(args.L, delta, j2)
    D = h.build_sector(NOD, (0, 0, 0))
    t0 = time.perf_counter()
    v = learned.start_vector(net, h, delta, j2)
    out["network"]["predict_s"] = time.perf_counter() - t0
    out["network"]["inference"] = mlp_inference_rate(net, h, D, delta, j2)
    if args.table:  # both arms read the cached connection table
        t0 = time.perf_counter()
        out["hv_table"] = {"bytes": h.hv_cache(True), "build_s": time.perf_counter() - t0}
    runs = [("learned_fp32_real", 1 | capi.REAL, v, 0.0)]
    if args.solve_all:
        runs += [("learned_fp32", 1, v, 0.0), ("random_fp32", 1, None, 0.0),
                 ("random_fp64_real", 0 | capi.REAL, None, 0.0), ("random_df", 2, None, 0.0)]
    runs.append(("plain_fp64_random", 0, None, args.plain_limit))
    psi = None
    for name, prec, start, limit in runs:
        h.set_time_limit(limit)
        t0 = time.perf_counter()
        r = h.trlan(1, args.nok, args.nom, maxitr=args.maxrestart, tol=args.tol, precision=prec, conv_mode=1,
                    seed=7, start=start, want_psi=psi is None, allow_unconverged=True)
        dt = time.perf_counter() - t0
        st = h.trlan_stats()
        if psi is None:
            psi = r["psi"][0]
            out["learned_start_overlap"] = float(abs(np.vdot(psi, v)) / np.linalg.norm(v))
        nhv = st["hv_fp32"] + st["hv_fp64"]
        out[name] = {"seconds": dt, "hv": r["iters"], "hv_fp32": st["hv_fp32"], "hv_fp64": st["hv_fp64"],
                     "fp32_share": st["hv_fp32"] / max(1, nhv), "restarts": st["restarts"],
                     "E0": float(r["ene"][0]), "resid": float(r["resid"][0]), "converged": bool(r["converged"]),
                     "timed_out": st["timed_out"], "ms_per_hv": 1e3 * dt / max(1, nhv)}
    h.set_time_limit(0.0)
    ref = out["plain_fp64_random"]
    for name, _, _, _ in runs:
        out[name]["dE_vs_plain_fp64"] = abs(out[name]["E0"] - ref["E0"])
    head = out["learned_fp32_real"]
    # a plain run stopped at its time limit gives a lower bound on the speed-up
    out["speedup_learned_fp32_real_vs_plain_fp64"] = ref["seconds"] / head["seconds"]
    out["speedup_is_lower_bound"] = bool(ref["timed_out"] or not ref["converged"])
    out["target_met"] = bool(head["converged"] and head["resid"] <= args.tol and
                             (out["speedup_is_lower_bound"] or head["dE_vs_plain_fp64"] <= 1e-10) and
                             out["speedup_learned_fp32_real_vs_plain_fp64"] >= 2.0)
    if args.solve_all:
        out["speedup_learned_fp32_vs_plain_fp64"] = ref["seconds"] / out["learned_fp32"]["seconds"]
        out["speedup_learned_vs_random_fp64_real"] = (out["random_fp64_real"]["seconds"] /
                                                      head["seconds"])
    out["sector_dim"] = D
    h.close()
    return out


def cfg5_bench(args):
    """The network's unseen test point (Delta = 0.7, J2 = 0.25: the Lifshitz
    point of the magnon band, where the k = 0 level spacing falls as L^-4) at
    L = 200 and L = 400, N_down = 4, k = 0: the learned start against the
    random start, both precision 1 with real vectors, to ||r|| <= tol, each
    solve stopped after --cfg5-limit seconds (reported, not converged)."""
    from ed_gb300 import capi, learned
    delta, j2 = 0.7, 0.25
    net = capi.Mlp(seed=1)
    learned.generate(net, learned.training_problems(seed=1))
    learned.train(net, rounds=10, steps=300, batch=4096, lr=2e-3)
    out = {"delta": delta, "J2": j2, "tol": args.tol, "NOK": args.nok, "NOM": args.nom,
           "limit_s": args.cfg5_limit}
    for L in (200, 400):
        h = learned.chain_handle(L, delta, j2)
        D = h.build_sector(NOD, (0, 0, 0))
        v = learned.start_vector(net, h, delta, j2)
        if args.table:
            h.hv_cache(True)
        rec = {"sector_dim": D}
        for name, start in (("learned", v), ("random", None)):
            h.set_time_limit(args.cfg5_limit)
            t0 = time.perf_counter()
            r = h.trlan(1, args.nok, args.nom, maxitr=args.maxrestart, tol=args.tol, precision=1 | capi.REAL,
                        conv_mode=1, seed=7, start=start, want_psi=(name == "learned"), allow_unconverged=True)
            dt = time.perf_counter() - t0
            st = h.trlan_stats()
            rec[name] = {"seconds": dt, "hv": r["iters"], "E0": float(r["ene"][0]), "resid": float(r["resid"][0]),
                         "converged": bool(r["converged"]), "timed_out": st["timed_out"]}
            if name == "learned":
                psi = r["psi"][0]
                rec["learned_start_overlap"] = float(abs(np.vdot(psi, v)) / np.linalg.norm(v) / np.linalg.norm(psi))
        h.set_time_limit(0.0)
        h.close()
        out[f"L{L}"] = rec
    return out


def batch_bench(args):
    """The batched-solve workload: 256 XXZ chains from seed 1 (L in
    {48..128}, N_down in {3, 4, 5}, k over the L momenta, Delta in [0, 2],
    J2 in [0, 0.5]), lowest 2 eigenpairs each to ||r|| <= 1e-10 with FP32
    Krylov vectors and FP64 reductions, from the same sectors:
      lockstep                   qs3g_trlan_lockstep: all problems in one
                                 graph-replayed launch sequence, row forms
                                 autotuned (it builds connection tables itself);
      batch_8_streams            qs3g_trlan_batch: each problem's own
                                 qs3g_trlan on its own stream, 8 host threads,
                                 matrix-free products;
      batch_8_streams_tables     the same with every sector's connection table
                                 cached first (qs3g_hv_cache)."""
    from ed_gb300 import sweep
    probs = sweep.random_chains(seed=1, n=args.batch_n)
    out = {"workload": f"{args.batch_n}_random_xxz_chains_L48-128_Ndown3-5_lowest2_tol1e-10_fp32_vectors",
           "NOE": 2, "NOK": 8, "NOM": 24}
    arms = [("lockstep", True, False), ("batch_8_streams", False, False)]
    if args.table:
        arms.append(("batch_8_streams_tables", False, True))
    e0 = None
    for name, lock, cache in arms:
        recs, tb, ts = sweep.solve(probs, NOE=2, NOK=8, NOM=24, tol=1e-10, precision=1, lockstep=lock,
                                   hv_cache=cache)
        out[name] = {"solve_s": ts, "build_s": tb, "all_ok": all(r["status"] == 0 for r in recs),
                     "max_resid": max(max(r["resid"]) for r in recs), "hv_total": sum(r["hv"] for r in recs)}
        out.setdefault("rows_total", sum(r["D"] for r in recs))
        if e0 is None:
            e0 = [r["ene"][0] for r in recs]
        else:
            out[name]["max_dE0_vs_lockstep"] = max(abs(a - r["ene"][0]) for a, r in zip(e0, recs))
    for name, _, _ in arms[1:]:
        out[f"speedup_lockstep_vs_{name}"] = out[name]["solve_s"] / out["lockstep"]["solve_s"]
    return out


def dsf_bench():
    """All q of a chain at once: L=200 Heisenberg ground state (N_down=3, k=0),
    S^-(q)|GS> in the N_down=4 sectors for q = 2 pi m / 200, m = 0..199, 150
    continued-fraction levels each, spectrum on 2000 omega points in [0, 6]
    with eta = 0.05; the same recursion one q at a time for comparison."""
    from ed_gb300 import capi, inputs
    L, nod, itr = 200, 3, 150
    b, jxy, jz = inputs.chain_bonds(L, (1.0, 1.0))
    h = capi.Handle(L, L, 1, 1, b, jxy, jz)
    h.build_sector(nod, (0, 0, 0))
    r = h.trlan(1, 8, 24, maxitr=5000, tol=1e-12, seed=3)
    psi, e0 = r["psi"][0], float(r["ene"][0])
    Spos = inputs.chain_positions(L)
    qs = [(2 * np.pi * m / L, 0.0, 0.0) for m in range(L)]
    h.dsf(psi, e0, 2, qs[:2], Spos, itr, 0.0)  # warm-up
    t0 = time.perf_counter()
    g = h.dsf(psi, e0, 2, qs, Spos, itr, 0.0)
    t_batch = time.perf_counter() - t0
    sample = list(range(0, L, 10))
    t0 = time.perf_counter()
    same = True
    for m in sample:
        one = h.dsf(psi, e0, 2, [qs[m]], Spos, itr, 0.0)
        same = same and np.array_equal(one["alpha"][0], g["alpha"][m]) and \
            np.array_equal(one["beta2"][0], g["beta2"][m])
    t_perq = (time.perf_counter() - t0) * L / len(sample)
    om = np.linspace(0.0, 6.0, 2000)
    t0 = time.perf_counter()
    S = capi.cfrac(g["alpha"], g["beta2"], g["nlev"], g["norm1"], g["E0"], 0.05, om, compat=True)
    t_cf = time.perf_counter() - t0
    h.close()
    return {"workload": "heisenberg_chain_L200_GS_Ndown3_Sminus_all_q_150_levels", "nq": L, "levels": itr,
            "batched_s": t_batch, "per_q_s_extrapolated": t_perq, "per_q_sample": len(sample),
            "speedup": t_perq / t_batch, "identical_to_per_q": bool(same), "cfrac_2000_omega_s": t_cf,
            "spectral_weight_finite": bool(np.isfinite(S[1:]).all())}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-solve", dest="solve", action="store_false",
                    help="skip the ground-state solves (learned start + anchored FP32 solver vs plain FP64 "
                         "random start; about 16 minutes, on by default)")
    ap.add_argument("--solve-all", action="store_true",
                    help="with the solves, also the complex-vector, random-start and real FP64 arms")
    ap.add_argument("--dsf", action="store_true", help="add the all-q DSF batch (L=200, 200 q, 150 levels)")
    ap.add_argument("--batch", action="store_true",
                    help="add the batched solves (256 random chains): lock step against concurrent streams")
    ap.add_argument("--batch-n", type=int, default=256, help="problems in --batch")
    ap.add_argument("--no-table", dest="table", action="store_false",
                    help="solves without the cached connection table (matrix-free H*v only)")
    ap.add_argument("--cfg5", action="store_true",
                    help="add the learned-vs-random start comparison at (Delta, J2) = (0.7, 0.25), L = 200 and 400")
    ap.add_argument("--cfg5-limit", type=float, default=300.0, help="wall seconds per --cfg5 solve")
    ap.add_argument("--nok", type=int, default=16)
    ap.add_argument("--nom", type=int, default=48)
    ap.add_argument("--maxrestart", type=int, default=40000)
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--arm", choices=sorted(ARMS), default=None,
                    help="run only this arm of the ground-state solve (no H*v leg) and print its line")
    ap.add_argument("--arm-limit", type=float, default=0.0, help="wall seconds for --arm (0: none)")
    ap.add_argument("--plain-limit", type=float, default=1200.0,
                    help="wall seconds after which the plain FP64 solve stops (reported as a lower bound)")
    ap.add_argument("--L", type=int, default=1000,
                    help="chain length (1000 is the benchmark; smaller sizes are for profiling)")
    return ap.parse_args()


def main():
    args = parse_args()
    global L_SITES, WORKLOAD
    if args.L != L_SITES:
        L_SITES = args.L
        WORKLOAD = WORKLOAD.replace("L1000", f"L{args.L}")
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local_rank, dist = dist_setup()
    try:
        if args.arm and rank == 0:
            solve_arm(args)
        elif args.arm:
            pass
        elif args.impl == "reference":
            run_reference(args, rank, world, dist)
        else:
            run_gpu(args, rank, world, local_rank, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
