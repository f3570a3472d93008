#!/usr/bin/env python
"""Benchmark of the fused extended-likelihood FdF on one GB300.

Workload (the production shape): the COMPASS 88-wave 3pi wave set -- 7
negative + 80 positive reflectivity waves + flat wave, rank 2 (341
parameters) -- over 1,000,000 synthetic data events stored as complex64
structure-of-arrays (696 MB, larger than the 129 MB L2, so no flush is needed
between steps), normalisation/acceptance integrals from 5,000,000 synthetic MC
events built on the GPU.  A step is one FdF (value + full gradient) at a new
parameter point.

  value     FdF evaluations per second with parameters and results resident in
            HBM (device-resident entry point, CUDA events on the launch stream)
  e2e       the same through the C ABI with host buffers (pwa_likelihood_fdf):
            every step copies the parameters host->device and the value and
            gradient device->host
  roofline  the fused event kernel: algorithmic bytes (N x W x 8) over its
            average launch duration in the timed region (CUDA events on the
            launch stream around the region, divided by the kernel launches
            in it: the fused kernel is the only kernel there), against the
            measured HBM copy bandwidth; the duration of a launch timed in
            isolation (events around each launch) is reported beside it
  cpu_baseline  the FP64 oracle (restatement of pwaLikelihood::FdF with the
            reference's compensated sums) on this machine's host cores

`--impl reference` times the reference's CPU FdF (the oracle restatement; the
reference itself cannot be built here) on all host threads instead.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_NEG, N_POS, RANK = 7, 80, 2
RANK_DEFAULT = RANK
METRIC = "FdF evals/s at 88 waves x 1M events"
UNIT = "FdF/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n-data", type=int, default=1_000_000)
    ap.add_argument("--store-block", type=int, default=0,
                    help="fdf: events per amplitude-store block and FdF tile (64 or 128; 0: automatic)")
    ap.add_argument("--shape", default="%d,%d,%d" % (N_NEG, N_POS, RANK),
                    help="fdf: negative waves, positive waves, rank (default: the production wave set)")
    ap.add_argument("--n-mc", type=int, default=5_000_000)
    ap.add_argument("--reduction", default="fp64", choices=["fp64", "kahan_fp32", "fp32"])
    ap.add_argument("--integral-precision", default="tf32x3", choices=["fp64", "fp32", "tf32", "tf32x3", "bf16x3"],
                    help="arithmetic of the normalisation / acceptance integrals (set-up, not timed)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sharded", action="store_true",
                    help="fdf: the event-sharded design (one all-reduce of P + 1 doubles per FdF) even on one "
                         "process (always on for more than one process)")
    ap.add_argument("--e2e-steps", type=int, default=0, help="steps of the host-buffer loop (default: min(steps, 2000))")
    ap.add_argument("--workload", default="fdf", choices=["fdf", "multibin", "precision", "next", "isobar", "config0"],
                    help="fdf: the headline FdF benchmark; multibin: whole multibin fit, plain multi-start vs "
                         "learned warm start; precision: error of each arithmetic variant against FP64; "
                         "isobar: decay amplitudes of the 88-wave 3pi set")
    ap.add_argument("--cross-tile-events", type=int, default=2_500_000,
                    help="precision: data events of the second cross-tile reduction comparison (several FP64 "
                         "folds per block; at 1 M events a block holds fewer tiles than one fold period)")
    ap.add_argument("--oracle-mc", type=int, default=200_000,
                    help="precision: MC events of the integrals compared with the CPU FP64 oracle")
    ap.add_argument("--bins", type=int, default=400, help="multibin: kinematic bins (100 mass x 4 t')")
    ap.add_argument("--starts", type=int, default=64, help="multibin: random start points of the plain fit")
    ap.add_argument("--train-bins", type=int, default=20_000, help="multibin: synthetic training bins")
    ap.add_argument("--augment", type=int, default=3, help="multibin: phase-rotated copies per training bin")
    ap.add_argument("--epochs", type=int, default=30, help="multibin: training epochs")
    ap.add_argument("--repeats", type=int, default=3, help="multibin: timed repeats of both fits (median reported)")
    ap.add_argument("--chunks", default="16,16,16",
                    help="multibin: tiles per work item for bins of < 64, < 512, >= 512 tiles (fixed, so that "
                         "repeats and runs take the same sweeps); 'auto' runs the chunk autotuner")
    ap.add_argument("--cpu-fits", type=int, default=4,
                    help="multibin: (bin, start) fits of the CPU baseline (scipy L-BFGS-B on the FP64 oracle)")
    ap.add_argument("--metrics-log", default=None,
                    help="also append the JSON line (with a UTC time stamp) to this JSON-lines file")
    ap.add_argument("--gtol-rel", type=float, default=1e-10,
                    help="multibin: L-BFGS stops when |grad| <= 1e-6 + gtol_rel * max(1, |f|)")
    return ap.parse_args()


def emit(line, args):
    """Prints the result line; with --metrics-log also appends it, time-stamped,
    to a JSON-lines metrics file."""
    print(json.dumps(line))
    if getattr(args, "metrics_log", None):
        rec = dict(line, time_utc=time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()))
        with open(args.metrics_log, "a") as f:
            f.write(json.dumps(rec) + "\n")


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per launch of the fused kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "fdf_main_compass88.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch:"):
            return float(line.split(":")[1])
    return None


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples while the GPU runs the workload."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.remove(self.path)
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, n in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def oracle_likelihood(names, refl, data_c64, mc_c64, accepted, rank):
    """FP64 oracle (the CPU restatement of the reference) on the given amplitudes."""
    from oracle.oracle import OracleIntegral, OracleLikelihood
    mc = mc_c64.astype(np.complex128)
    norm, acc = OracleIntegral(), OracleIntegral()
    assert norm.integrate(names, mc) and acc.integrate(names, mc, in_bin=accepted)
    L = OracleLikelihood()
    assert L.init(names, refl, None, rank, 0.0)
    assert L.addNormIntegral(norm) and L.addAccIntegral(acc)
    for k, n in enumerate(names):
        assert L.addAmplitude(n, data_c64[k].astype(np.complex128))
    assert L.finishInit()
    return L


def integral_snapshot(I):
    """(wave names, raw sums, event count) of a product integral"""
    return I.waveNames(), I.matrix(), I.nmbEvents()


def oracle_with_integrals(names, refl, data_c64, norm, acc, rank, shard=None):
    """FP64 oracle on the given data amplitudes with exactly the raw sums and
    event counts of the product's normalisation and acceptance integrals
    (integral_snapshot, taken before addAccIntegral changes the acceptance
    integral's event count), so that a comparison of the two likelihoods
    measures the event term alone."""
    from oracle.oracle import OracleIntegral, OracleLikelihood
    ints = []
    for wn, raw, n in (norm, acc):
        o = OracleIntegral()
        assert o.set_wave_names(wn)
        o.set_raw(raw)
        o.set_nmb_events(n)
        ints.append(o)
    L = OracleLikelihood()
    if shard is not None:
        L.set_shard(*shard)
    assert L.init(names, refl, None, rank, 0.0)
    assert L.addNormIntegral(ints[0]) and L.addAccIntegral(ints[1])
    for k, n in enumerate(names):
        assert L.addAmplitude(n, data_c64[k].astype(np.complex128))
    assert L.finishInit()
    return L


def time_oracle(L, par, threads, min_seconds, max_reps):
    """Median seconds of one oracle FdF."""
    ts = []
    t_start = time.perf_counter()
    while len(ts) < max_reps and (len(ts) < 1 or time.perf_counter() - t_start < min_seconds):
        t0 = time.perf_counter()
        L.FdF(par, threads=threads)
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts), len(ts)


def run_reference(args):
    """--impl reference: the reference's CPU FdF (oracle restatement) on all host threads."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from rootpwa_gb300 import synth
    names, refl = synth.wave_names(N_NEG, N_POS)
    rng = np.random.Generator(np.random.PCG64(1))
    model = synth.AmplitudeModel(len(names), 8, rng)
    par = rng.standard_normal(synth.n_pars(N_NEG, N_POS, RANK))
    threads = cpu_threads()
    # size the per-step event sample so that warm-up + steps take about two minutes
    calib = model.draw(rng, 20_000)
    mc = model.draw(rng, 20_000)
    acc = rng.random(20_000) < 0.6
    Lc = oracle_likelihood(names, refl, calib, mc, acc, RANK)
    t_cal, _ = time_oracle(Lc, par, threads, 0.5, 5)
    per_event = t_cal / 20_000
    budget = 120.0
    n_sample = int(budget / max(1, args.steps + args.warmup) / per_event)
    n_sample = max(20_000, min(args.n_data, n_sample))
    data = model.draw(rng, n_sample)
    L = oracle_likelihood(names, refl, data, mc, acc, RANK)
    for _ in range(args.warmup):
        L.FdF(par, threads=threads)
    ts = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        L.FdF(par * (1.0 + 1e-3 * (k % 7)), threads=threads)
        ts.append(time.perf_counter() - t0)
    t_step = sum(ts) / len(ts)
    value = 1.0 / (t_step * args.n_data / n_sample)
    sample = ("FP64 oracle FdF (restatement of pwaLikelihood::FdF, compensated sums) over %d of the %d events "
              "per step on %d host threads, scaled to %d events" % (n_sample, args.n_data, threads, args.n_data))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3 * args.n_data / n_sample,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "compass88: 7-/80+ waves + flat, rank 2, %d events" % args.n_data,
                       "waves": 88, "rank": RANK, "events": args.n_data, "parameters": len(par)},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    emit(line, args)
    return 0


def run_gb300(args):
    import torch
    rank, world, local = dist_env()
    sharded = args.sharded or world > 1
    torch.cuda.set_device(local)
    if sharded:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import rootpwa_gb300 as R
    from rootpwa_gb300 import synth
    from rootpwa_gb300 import _native as N

    n_neg, n_pos, RANK = (int(v) for v in args.shape.split(","))
    names, refl = synth.wave_names(n_neg, n_pos)
    W = len(names)
    rng = np.random.Generator(np.random.PCG64(1))
    model = synth.AmplitudeModel(W, 8, rng)
    P = synth.n_pars(n_neg, n_pos, RANK)
    default_shape = (n_neg, n_pos, RANK) == (N_NEG, N_POS, RANK_DEFAULT)
    metric = METRIC if default_shape else "FdF evals/s at %d waves x %d events" % (W + 1, args.n_data)
    par0 = rng.standard_normal(P)

    # ---- set-up (not timed): amplitudes on the device, integrals on the GPU ----
    data = synth.draw_device(model, args.n_data, seed=11 + rank)
    mc = synth.draw_device(model, args.n_mc, seed=1011 + rank)
    g = torch.Generator(device="cuda")
    g.manual_seed(2011 + rank)
    accepted = (torch.rand(args.n_mc, generator=g, device="cuda") < 0.6).to(torch.uint8).cpu().numpy()
    torch.cuda.synchronize()
    # the tensor-core Gram covers up to 128 waves; wider sets use the SIMT FP32 kernel
    int_prec = args.integral_precision if W <= 128 or args.integral_precision in ("fp32", "fp64") else "fp32"
    t0 = time.perf_counter()
    norm = R.ampIntegralMatrix()
    norm.integrate(names, mc, precision=int_prec)
    integral_s = time.perf_counter() - t0
    acc = R.ampIntegralMatrix()
    acc.integrate(names, mc, inBin=accepted, precision=int_prec)
    if sharded:
        # every rank integrated its own MC events: one all-reduce of the raw
        # sums and event counts gives every rank the integrals of all of them
        for I in (norm, acc):
            raw = torch.from_numpy(np.ascontiguousarray(I.matrix()).view(np.float64).copy()).cuda()
            cnt = torch.tensor([float(I.nmbEvents())], dtype=torch.float64, device="cuda")
            dist.all_reduce(raw)
            dist.all_reduce(cnt)
            I.setMatrix(raw.cpu().numpy().view(np.complex128).reshape(W, W))
            I.setNmbEvents(int(round(cnt.item())))
    int_snap = (integral_snapshot(norm), integral_snapshot(acc))
    del mc
    torch.cuda.empty_cache()
    L = R.pwaLikelihood()
    if args.store_block:
        L.setStoreBlock(args.store_block)
    if sharded:
        # this rank's share of a data set of world x n_data events: only the
        # root shard adds the normalisation and prior terms
        L.setShard(world * args.n_data, rank == 0)
    L.init(names, refl, None, RANK, 0.0)
    L.addNormIntegral(norm)
    L.addAccIntegral(acc)
    for k, n in enumerate(names):
        L.addAmplitude(n, data[k])
    L.finishInit()
    L.setReduction(args.reduction)
    stream = torch.cuda.Stream()
    L.setStream(stream.cuda_stream)

    # distinct parameter points, resident in HBM
    n_pts = 64
    pts = np.stack([par0 * (1.0 + 0.01 * k) for k in range(n_pts)])
    d_par = torch.from_numpy(pts).cuda()
    d_out = torch.zeros((n_pts, P + 2), dtype=torch.float64, device="cuda")
    par_ptr = [d_par[k].data_ptr() for k in range(n_pts)]
    out_ptr = [d_out[k].data_ptr() for k in range(n_pts)]
    lib = N.lib()
    h = L._h
    fdf_dev = lib.pwa_likelihood_fdf_device
    sptr = C.c_void_p(stream.cuda_stream)

    def step(i):
        st = fdf_dev(h, C.c_void_p(par_ptr[i % n_pts]), C.c_void_p(out_ptr[i % n_pts]), 1, sptr)
        if st:
            N.check(st)
        if sharded:
            # f and the gradient of all shards, on the kernel's stream
            with torch.cuda.stream(stream):
                dist.all_reduce(d_out[i % n_pts, :P + 1])

    for i in range(max(3, args.warmup)):
        step(i)
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    # keep the GPU busy for about a second before the timed region so that
    # the clock samples describe the sustained state of this workload
    t_pre = time.perf_counter()
    i = 0
    while time.perf_counter() - t_pre < 1.0:
        step(i)
        i += 1
        if i % 200 == 0:
            stream.synchronize()
    stream.synchronize()
    launches0 = lib.pwa_kernel_launch_count()
    if sharded:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for i in range(args.steps):
        step(i)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    launches = lib.pwa_kernel_launch_count() - launches0
    ms = ev0.elapsed_time(ev1)
    # the same steps once more with CUDA events around each of the two
    # kernels (on the launch stream) for the per-kernel durations
    L.setTiming(True)
    for i in range(args.steps):
        step(i)
    main_ms, fin_ms, n_timed = L.kernelTimes()
    L.setTiming(False)
    clocks = sampler.stop()
    out = d_out.cpu().numpy()
    assert np.all(out[:, P + 1] == 0.0), "device error flag set"
    assert np.all(np.isfinite(out[:, :P + 1]))
    if sharded:
        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = world * args.steps / (ms / 1e3)

    # cross-check the device-resident result against the host entry point
    # (in the sharded design: the host-API ShardedFdF over all ranks)
    if sharded:
        from rootpwa_gb300.sharded import ShardedFdF
        whole = ShardedFdF(L, device="cuda")
        f_host, g_host = whole.FdF(pts[0])
    else:
        f_host, g_host = L.FdF(pts[0])
    f_dev = out[0, 0]
    assert abs(f_dev - f_host) <= 1e-12 * abs(f_host), (f_dev, f_host)

    # ---- e2e: the C-ABI call with host buffers (sharded: the ShardedFdF
    # host API, whose all-reduce buffer goes host -> device -> host) ----
    n_e2e = args.e2e_steps or min(args.steps, 2000)
    host_pts = [np.ascontiguousarray(p) for p in pts]
    fbuf = C.c_double()
    gbuf = np.zeros(P)
    gptr = gbuf.ctypes.data_as(C.POINTER(C.c_double))
    pptrs = [p.ctypes.data_as(C.POINTER(C.c_double)) for p in host_pts]
    fdf_host = lib.pwa_likelihood_fdf

    def e2e_step(i):
        if sharded:
            whole.FdF(host_pts[i % n_pts])
            return
        st = fdf_host(h, pptrs[i % n_pts], C.byref(fbuf), gptr)
        if st:
            N.check(st)

    for i in range(3):
        e2e_step(i)
    if sharded:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for i in range(n_e2e):
        e2e_step(i)
    e2e_s = time.perf_counter() - t0
    if sharded:
        t = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * n_e2e / e2e_s

    # ---- roofline of the fused event kernel ----
    alg_bytes = args.n_data * W * 8
    avg_main_s = ms / 1e3 / max(1, launches)
    isolated_s = main_ms / max(1, n_timed) / 1e3
    achieved = alg_bytes / avg_main_s / 1e9
    peak, peak_kind = measured_peaks()
    roofline = {"bound": "hbm", "kernel": "fdfMainKernel", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": profile_traffic() if default_shape else None,
                "algorithmic_bytes_per_launch": alg_bytes, "avg_launch_us": avg_main_s * 1e6,
                "isolated_launch_us": isolated_s * 1e6,
                "frac_isolated_launch": alg_bytes / isolated_s / 1e9 / peak,
                "frac_of_8TBs_spec": achieved / 8000.0}

    # ---- parity and CPU baseline: the FP64 oracle on this machine's host cores,
    # over the same events, with the product's own integral sums (sharded:
    # every rank's oracle over its shard, summed like the product's) ----
    cpu = parity = None
    if rank == 0 or sharded:
        n_cpu = args.n_data
        host = data[:, :n_cpu].cpu().numpy()
        Lo = oracle_with_integrals(names, refl, host, int_snap[0], int_snap[1], RANK,
                                   shard=(world * args.n_data, rank == 0) if sharded else None)
        del host
        threads = cpu_threads()
        f_o, g_o = Lo.FdF(pts[0], threads=threads)
        if sharded:
            buf = torch.from_numpy(np.concatenate([[f_o], g_o])).cuda()
            torch.distributed.all_reduce(buf)
            buf = buf.cpu().numpy()
            f_o, g_o = float(buf[0]), buf[1:]
    if rank == 0:
        ll_rel = abs(f_host - f_o) / abs(f_o)
        parity = {"ll_rel": ll_rel, "grad_normwise": float(np.max(np.abs(g_host - g_o)) / np.max(np.abs(g_o))),
                  "events": world * n_cpu if sharded else n_cpu, "point": "pts[0]", "tolerance_ll_rel": 1e-6,
                  "against": "FP64 oracle (bit-for-bit restatement of pwaLikelihood::FdF) with the same "
                             "normalisation and acceptance sums"}
        if not ll_rel <= 1e-6:
            raise SystemExit("parity failure at full size: ll_rel %.3g > 1e-6" % ll_rel)
        if not args.no_cpu_baseline:
            t_all, reps_all = time_oracle(Lo, pts[0], threads, 8.0, 10)
            t_one, reps_one = time_oracle(Lo, pts[0], 1, 0.0, 1)
            cpu = {"value": 1.0 / t_all, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": ("FP64 oracle FdF over all %d events (%d reps, median) on %d host threads; "
                              "single-thread (the reference is single-threaded): %.4f FdF/s" %
                              (n_cpu, reps_all, threads, 1.0 / t_one)),
                   "single_thread_value": 1.0 / t_one}

    if rank == 0:
        line = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32 (complex64 store, FP64 cross-tile reductions)",
                "data": "synthetic",
                "config": {"workload": ("compass88: 7-/80+ waves + flat, rank 2, %d events per GPU" % args.n_data
                                        if default_shape else "%d-/%d+ waves + flat, rank %d, %d events per GPU"
                                        % (n_neg, n_pos, RANK, args.n_data)),
                           "waves": W + 1, "rank": RANK, "events": args.n_data, "parameters": P,
                           "mc_events": args.n_mc, "reduction": args.reduction,
                           "l2": "inputs (%.0f MB) larger than L2 (129 MB); no flush" % (alg_bytes / 1e6),
                           "entry": "pwa_likelihood_fdf_device (parameters and results in HBM)",
                           "design": ("event-sharded: rank r holds events [r n, (r+1) n) of one data set of "
                                      "%d x %d events; per FdF one NCCL all-reduce of P + 1 doubles on the "
                                      "kernel's stream; value counts %d-event FdF equivalents"
                                      % (world, args.n_data, args.n_data)) if sharded else
                                     "one process, one likelihood",
                           "plan": dict(zip(("tile_events", "stages", "blocks"), L.plan()),
                                        phase1_events_per_lane=L.planVariant())},
                "e2e": {"value": e2e_value, "unit": UNIT,
                        "h2d_bytes_per_step": P * 8 + ((P + 1) * 8 if sharded else 0),
                        "d2h_bytes_per_step": (P + 2) * 8 + ((P + 1) * 8 if sharded else 0),
                        "entry": ("rootpwa_gb300.sharded.ShardedFdF.FdF (host parameters; per rank "
                                  "pwa_likelihood_fdf of its shard, then one NCCL all-reduce of P + 1 doubles)"
                                  if sharded else
                                  "pwa_likelihood_fdf (host buffers, staged through mapped pinned memory that "
                                  "the kernel reads and writes directly)")},
                "gpu_launches": int(launches), "launches_per_step": launches / args.steps,
                "roofline": roofline, "cpu_baseline": cpu, "parity": parity, "clocks": clocks,
                "extra": {"integral_norm_s": integral_s, "integral_precision": int_prec,
                          "mc_events": args.n_mc}}
        emit(line, args)
    if sharded:
        torch.distributed.destroy_process_group()
    return 0


def run_multibin(args):
    """Whole multibin fit (100 mass x 4 t' bins, 50 positive-reflectivity waves
    + flat, rank 1): the plain fit from `starts` random start points per bin
    against the learned warm start (moments -> network -> 1 warm + 4 random
    start points), both refined by the batched GPU L-BFGS.  Data of each bin
    follow the model intensity of known amplitudes; normalisation and
    acceptance integrals from 5x as many phase-space events per bin."""
    import torch
    import rootpwa_gb300 as R
    from rootpwa_gb300 import synth
    from rootpwa_gb300 import warmstart as WS
    W = 50
    names, _ = synth.wave_names(0, W)
    counts = synth.multibin_event_counts(n_bins=args.bins, seed=0)
    model = synth.AmplitudeModel(W, 0, np.random.Generator(np.random.PCG64(5)))
    rng = np.random.default_rng(1)
    torch.cuda.synchronize()
    t_setup = time.perf_counter()
    bins = []
    for b, n in enumerate(counts):
        n = int(n)
        vt, fl = synth.true_production_amplitudes(W, rng)
        data = synth.draw_bin_device(model, vt, fl, n, seed=1000 + b)
        mc = synth.draw_device(model, 5 * n, seed=2_000_000 + b)
        g = torch.Generator(device="cuda")
        g.manual_seed(3_000_000 + b)
        accepted = (torch.rand(5 * n, generator=g, device="cuda") < 0.6).to(torch.uint8).cpu().numpy()
        norm = R.ampIntegralMatrix()
        norm.integrate(names, mc, precision="tf32x3")
        acc = R.ampIntegralMatrix()
        acc.integrate(names, mc, inBin=accepted, precision="tf32x3")
        del mc
        diag = np.real(np.diag(norm.matrix())) / norm.nmbEvents()
        ints = (integral_snapshot(norm), integral_snapshot(acc))
        L = R.pwaLikelihood()
        L.init(names, [1] * W, None, 1, 0.0)
        L.addNormIntegral(norm)
        L.addAccIntegral(acc)
        for k, nm in enumerate(names):
            L.addAmplitude(nm, data[k])
        L.finishInit()
        bins.append(dict(L=L, n=n, data=data, diag=diag, ints=ints))
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t_setup
    P = bins[0]["L"].nmbPars()

    # ---- training set (method-generated pairs) and network training ----
    t0 = time.perf_counter()
    tmc = synth.draw_device(model, 4_000_000, seed=77)
    tnorm = R.ampIntegralMatrix()
    tnorm.integrate(names, tmc, precision="tf32x3")
    tacc = R.ampIntegralMatrix()
    tacc.integrate(names, tmc, inBin=(torch.rand(4_000_000, device="cuda") < 0.6).to(torch.uint8).cpu().numpy(),
                   precision="tf32x3")
    del tmc
    tcounts = synth.multibin_event_counts(n_bins=args.train_bins, seed=11)

    def draw_bin(vt, fl, n, k):
        return synth.draw_bin_device(model, vt, fl, n, seed=10_000_000 + k)

    F, Y, _ = WS.generate_training_set(names, draw_bin, tnorm, tacc, tcounts, np.random.default_rng(12), chunk=500)
    gen_s = time.perf_counter() - t0
    Fa, Ya = WS.augment_phases(F, Y, W, args.augment, np.random.default_rng(13))
    t0 = time.perf_counter()
    net = R.pwaMLP(Fa.shape[1], 512, 512, Ya.shape[1], seed=14)
    net.fit_standardisation(Fa)
    hist = net.train(net.standardise(Fa), Ya, batch=256, epochs=args.epochs, lr=1e-3)
    train_s = time.perf_counter() - t0
    del Fa, Ya

    # ---- plain multi-start fit ----
    S = args.starts
    Mp = R.pwaMultibin()
    Mp.setOptions(startGroup=32 if S > 8 else 8, gtolAbs=1e-6, gtolRel=args.gtol_rel, maxIter=5000)
    for bn in bins:
        Mp.addBin(bn["L"], S)
    x0 = np.random.default_rng(21).standard_normal((len(bins) * S, P))
    fixed_chunks = None if args.chunks == "auto" else [int(c) for c in args.chunks.split(",")]

    def set_chunks(M, x):
        if fixed_chunks is None:
            return M.autotune(x)
        M.setChunks(fixed_chunks)
        return fixed_chunks

    chunks_plain = set_chunks(Mp, x0)
    sweep_ms = Mp.sweepMs(x0)
    plain_runs = []
    for _ in range(max(1, args.repeats)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rp = Mp.fit(x0, sweepsPerGraph=10)
        torch.cuda.synchronize()
        plain_runs.append((time.perf_counter() - t0, rp["sweeps"], Mp.trace()))
    plain_s = float(np.median([r[0] for r in plain_runs]))

    # ---- learned warm start: features + inference + 1 warm + 4 random starts ----
    Sw = 5
    Mw = R.pwaMultibin()
    Mw.setOptions(startGroup=8, gtolAbs=1e-6, gtolRel=args.gtol_rel, maxIter=5000)
    for bn in bins:
        Mw.addBin(bn["L"], Sw)
    xr = np.random.default_rng(22).standard_normal((len(bins) * Sw, P))
    chunks_learned = set_chunks(Mw, xr)
    # one-time kernel loading of the feature and inference paths, outside the timed region
    WS.moment_features_batch([bins[0]["data"]], [bins[0]["diag"]])
    net.forward(np.zeros((1, net.shape[0]), dtype=np.float32))
    learned_runs = []
    for _ in range(max(1, args.repeats)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Fe = WS.moment_features_batch([bn["data"] for bn in bins], [bn["diag"] for bn in bins])
        t_feat = time.perf_counter()
        Yp = net.forward(net.standardise(Fe))
        xw = xr.copy()
        for b, bn in enumerate(bins):
            xw[b * Sw] = WS.params_from_targets(bn["L"], Yp[b], bn["n"])
        t_inf = time.perf_counter()
        rw = Mw.fit(xw, sweepsPerGraph=10)
        torch.cuda.synchronize()
        t_end = time.perf_counter()
        learned_runs.append((t_end - t0, rw["sweeps"], Mw.trace(),
                             {"features_s": t_feat - t0, "inference_s": t_inf - t_feat, "fit_s": t_end - t_inf}))
    k_med = int(np.argsort([r[0] for r in learned_runs])[len(learned_runs) // 2])
    learned_s = learned_runs[k_med][0]
    breakdown = learned_runs[k_med][3]

    fp = rp["f"].reshape(len(bins), S)
    fw = rw["f"].reshape(len(bins), Sw)
    fstar = np.minimum(fp.min(axis=1), fw.min(axis=1))
    tol = 1e-6 * np.abs(fstar)

    def time_to_global(trace, starts, offset):
        # first check at which every bin has a start within 1e-6 of its global minimum
        t, f = trace
        for k in range(len(t)):
            best = np.nanmin(f[k].reshape(len(bins), starts), axis=1)
            if np.all(best <= fstar + tol):
                return offset + float(t[k])
        return None

    ttg_p = [time_to_global(r[2], S, 0.0) for r in plain_runs]
    ttg_w = [time_to_global(r[2], Sw, r[3]["features_s"] + r[3]["inference_s"]) for r in learned_runs]
    ttg_plain = float(np.median(ttg_p)) if all(v is not None for v in ttg_p) else None
    ttg_learned = float(np.median(ttg_w)) if all(v is not None for v in ttg_w) else None
    reach_p = float(np.mean(fp.min(axis=1) <= fstar + tol))
    reach_w = float(np.mean(fw.min(axis=1) <= fstar + tol))
    warm_alone = float(np.mean(fw[:, 0] <= fstar + tol))
    # fitted-V agreement in units of the parameter errors (Hessian of 16 bins)
    verr = []
    for b in range(0, len(bins), max(1, len(bins) // 16)):
        L = bins[b]["L"]
        xa = L.CorrectParamSigns(rp["x"][b * S + int(np.argmin(fp[b]))])
        xb = L.CorrectParamSigns(rw["x"][b * Sw + int(np.argmin(fw[b]))])
        if abs(fp[b].min() - fw[b].min()) > tol[b]:
            continue
        cov = L.CovarianceMatrix(xa)
        sig = np.sqrt(np.maximum(np.diag(cov), 1e-300))
        verr.append(float(np.max(np.abs(xa - xb) / sig)))
    # ---- roofline of one full sweep of the plain fit (all problems active):
    # each tile is read once per group of `group` starts; 16 flop per
    # (event, start, wave) (value and gradient contractions, complex FMA) ----
    group = 32 if S > 8 else 8
    n_tot = int(counts.sum())
    sweep_bytes = n_tot * W * 8 * ((S + group - 1) // group)
    sweep_flop = 16.0 * n_tot * S * W
    hbm_peak, peak_kind = measured_peaks()
    fp32_nominal = 152 * 128 * 2 * 2.07e9 / 1e12  # SIMT FP32 FMA lanes x 2 flop x max SM clock
    sweep_roofline = {"bound": "fp32 simt", "achieved": sweep_flop / (sweep_ms / 1e3) / 1e12,
                      "peak": fp32_nominal, "unit": "TFLOP/s",
                      "frac": sweep_flop / (sweep_ms / 1e3) / 1e12 / fp32_nominal,
                      "peak_source": "nominal (152 SMs x 128 FP32 lanes x 2 flop x 2.07 GHz); not measured",
                      "hbm_achieved_gbs": sweep_bytes / (sweep_ms / 1e3) / 1e9, "hbm_peak_gbs": hbm_peak,
                      "hbm_frac": sweep_bytes / (sweep_ms / 1e3) / 1e9 / hbm_peak,
                      "algorithmic_bytes_per_sweep": sweep_bytes, "algorithmic_flop_per_sweep": sweep_flop,
                      "sweep_ms": sweep_ms}

    # ---- CPU baseline: scipy L-BFGS-B on the FP64 oracle (the reference's
    # likelihood arithmetic) for a sample of (bin, start) fits, extrapolated
    # to every bin and start in proportion to the bin's events ----
    cpu = None
    if args.cpu_fits > 0:
        import scipy.optimize as so
        threads = cpu_threads()
        # bins spread over the event-count distribution (quantiles)
        order = np.argsort(counts)
        pick = [int(order[(2 * i + 1) * len(order) // (2 * args.cpu_fits)]) for i in range(args.cpu_fits)]
        fit_s, fit_ev, nfev = [], [], []
        for b in pick:
            bn = bins[b]
            Lo = oracle_with_integrals(names, [1] * W, bn["data"].cpu().numpy(), bn["ints"][0], bn["ints"][1], 1)
            xs = x0[b * S]
            t_c = time.perf_counter()
            r = so.minimize(lambda p: Lo.FdF(p, threads=threads), xs, jac=True, method="L-BFGS-B",
                            options=dict(maxiter=5000, gtol=1e-6, ftol=1e-15))
            fit_s.append(time.perf_counter() - t_c)
            fit_ev.append(bn["n"])
            nfev.append(int(r.nfev))
        per_event_fit = float(np.sum(fit_s) / np.sum(fit_ev))
        total = per_event_fit * n_tot * S
        cpu = {"value": total, "unit": "s", "cores": threads, "kind": "port",
               "sample": ("%d (bin, start) fits (bins of %s events; %s FdF evaluations) with scipy L-BFGS-B "
                          "(gtol 1e-6) on the FP64 oracle on %d host threads took %.1f s; extrapolated to %d bins "
                          "x %d starts in proportion to events (%.3g s per event and start)"
                          % (len(pick), [int(e) for e in fit_ev], nfev, threads, float(np.sum(fit_s)), len(bins), S,
                             per_event_fit)),
               "compares_to": "full_fit_s.plain"}

    line = {"metric": "multibin fit: GPU wall time to reach every bin's global-minimum LL (1e-6 relative), "
                      "learned warm start", "value": ttg_learned, "unit": "s", "higher_is_better": False,
            "n_gpus": 1, "impl": "gb300",
            "plain_time_to_global_s": ttg_plain,
            "speedup_time_to_global": (ttg_plain / ttg_learned) if (ttg_plain and ttg_learned) else None,
            "full_fit_s": {"learned": learned_s, "plain": plain_s, "speedup": plain_s / learned_s,
                           "statistic": "median of %d repeats" % len(plain_runs),
                           "plain_runs": [r[0] for r in plain_runs], "learned_runs": [r[0] for r in learned_runs]},
            "time_to_global_runs_s": {"plain": ttg_p, "learned": ttg_w},
            "learned_breakdown": breakdown,
            "roofline_sweep": sweep_roofline, "cpu_baseline": cpu,
            "chunks": {"plain": list(chunks_plain), "learned": list(chunks_learned),
                       "mode": "autotuned" if fixed_chunks is None else "fixed"},
            "data": "synthetic",
            "config": {"workload": "%d bins x 50 waves + flat, rank 1, %d data events (log-normal per bin), "
                                   "MC 5x per bin" % (len(bins), int(counts.sum())),
                       "starts_plain": S, "starts_learned": Sw, "gtol": "1e-6 + %g x max(1, |f|)" % args.gtol_rel,
                       "network": "5203-512-512-102 BF16/FP32, %d training bins x %d copies, %d epochs" %
                                  (args.train_bins, args.augment + 1, args.epochs)},
            "reached_global_min": {"plain": reach_p, "learned": reach_w, "warm_start_alone": warm_alone},
            "v_error_sigma_max": max(verr) if verr else None, "v_error_bins": len(verr),
            "sweeps": {"plain": [r[1] for r in plain_runs], "learned": [r[1] for r in learned_runs]},
            "full_sweep_ms_plain": sweep_ms,
            "status_counts": {"plain": np.bincount(rp["status"], minlength=7).tolist(),
                              "learned": np.bincount(rw["status"], minlength=7).tolist(),
                              "order": ["active", "searching", "converged", "max_iter", "stalled", "failed",
                                        "floor"]},
            "training": {"generate_s": gen_s, "train_s": train_s, "loss_first": float(hist[0]),
                         "loss_last": float(hist[-1])},
            "setup_s": setup_s}
    emit(line, args)
    return 0


def run_precision(args):
    """Precision sweep on the production shapes (87 waves + flat, rank 2): the
    integral matrix in FP64 / FP32 (SIMT) / TF32 / TF32x3 (tensor cores), the
    FdF with FP64, compensated-FP32 or plain FP32 cross-tile reductions, and the effect of
    each integral variant on LL and gradient; errors against FP64 (the CPU
    oracle, and the GPU FP64 kernels at full size)."""
    import torch
    import rootpwa_gb300 as R
    from rootpwa_gb300 import synth
    from oracle.oracle import OracleIntegral, OracleLikelihood
    names, refl = synth.wave_names(N_NEG, N_POS)
    W = len(names)
    rng = np.random.Generator(np.random.PCG64(1))
    model = synth.AmplitudeModel(W, 8, rng)
    P = synth.n_pars(N_NEG, N_POS, RANK)
    par = rng.standard_normal(P)
    precs = ["fp32", "tf32", "tf32x3", "bf16x3"]

    def maxrel(a, b):
        return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))

    out = {}
    # integrals against the CPU FP64 oracle (smaller MC sample)
    mcs = model.draw(np.random.Generator(np.random.PCG64(2)), args.oracle_mc)
    oi = OracleIntegral()
    assert oi.integrate(names, mcs.astype(np.complex128))
    ref = oi.raw()
    out["integral_vs_oracle"] = {"mc_events": args.oracle_mc}
    for p in ["fp64"] + precs:
        I = R.ampIntegralMatrix()
        I.integrate(names, mcs, precision=p)
        out["integral_vs_oracle"][p] = maxrel(I.matrix(), ref)
    # integrals at full size against the GPU FP64 kernel
    mc = synth.draw_device(model, args.n_mc, seed=1011)
    ints = {}
    out["integral_ms"] = {"mc_events": args.n_mc, "timing": "host-timed integrate() of device-resident "
                          "amplitudes, best of 3 after one warm-up call"}
    for p in ["fp64"] + precs:
        I = R.ampIntegralMatrix()
        I.integrate(names, mc, precision=p)
        ints[p] = I
        best = 1e30
        for _ in range(3):
            J = R.ampIntegralMatrix()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            J.integrate(names, mc, precision=p)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        out["integral_ms"][p] = best * 1e3
    out["integral_vs_fp64"] = {"mc_events": args.n_mc}
    for p in precs:
        out["integral_vs_fp64"][p] = maxrel(ints[p].matrix(), ints["fp64"].matrix())
    g = torch.Generator(device="cuda")
    g.manual_seed(2011)
    accepted = (torch.rand(args.n_mc, generator=g, device="cuda") < 0.6).to(torch.uint8).cpu().numpy()
    accs = {}
    for p in ["fp64"] + precs:
        J = R.ampIntegralMatrix()
        J.integrate(names, mc, inBin=accepted, precision=p)
        accs[p] = J
    del mc
    data = synth.draw_device(model, args.n_data, seed=11)
    host = data.cpu().numpy()

    def copy(I):
        C_ = R.ampIntegralMatrix(I)
        return C_

    def oracle_copy(I):
        o = OracleIntegral()
        o.set_wave_names(I.waveNames())
        o.set_raw(I.matrix())
        o.set_nmb_events(I.nmbEvents())
        return o

    # FP64 oracle likelihood with the FP64 integrals
    O = OracleLikelihood()
    assert O.init(names, refl, None, RANK, 0.0)
    assert O.addNormIntegral(oracle_copy(ints["fp64"])) and O.addAccIntegral(oracle_copy(accs["fp64"]))
    for k, n in enumerate(names):
        assert O.addAmplitude(n, host[k].astype(np.complex128))
    assert O.finishInit()
    f0, g0 = O.FdF(par, threads=cpu_threads())
    def cross_tile(key, dev_data, nev, fref, gref):
        out[key] = {"events": nev, "tiles_per_block": round(nev / 128 / 152, 1)}
        for red in ["fp64", "kahan_fp32", "fp32"]:
            L = R.pwaLikelihood()
            L.init(names, refl, None, RANK, 0.0)
            L.addNormIntegral(copy(ints["fp64"]))
            L.addAccIntegral(copy(accs["fp64"]))
            for k, n in enumerate(names):
                L.addAmplitude(n, dev_data[k])
            L.finishInit()
            L.setReduction(red)
            f, gg = L.FdF(par)
            for _ in range(5):
                L.FdF(par)
            t0 = time.perf_counter()
            for _ in range(100):
                L.FdF(par)
            us = (time.perf_counter() - t0) / 100 * 1e6
            out[key][red] = {"ll_rel": abs(f - fref) / abs(fref),
                             "grad_normwise": float(np.max(np.abs(gg - gref)) / np.max(np.abs(gref))),
                             "us_per_fdf_host_call": us,
                             "cross_tile": {"fp64": "FP32 partials of 64 tiles folded into FP64",
                                            "kahan_fp32": "every tile into compensated FP32",
                                            "fp32": "plain FP32 over all tiles"}[red]}

    cross_tile("fdf_vs_oracle", data, args.n_data, f0, g0)
    # a larger set: each block folds its FP32 partials into FP64 more than once
    if args.cross_tile_events > args.n_data:
        data2 = synth.draw_device(model, args.cross_tile_events, seed=12)
        O2 = OracleLikelihood()
        assert O2.init(names, refl, None, RANK, 0.0)
        assert O2.addNormIntegral(oracle_copy(ints["fp64"])) and O2.addAccIntegral(oracle_copy(accs["fp64"]))
        for k, n in enumerate(names):
            assert O2.addAmplitude(n, data2[k].cpu().numpy().astype(np.complex128))
        assert O2.finishInit()
        f2, g2 = O2.FdF(par, threads=cpu_threads())
        del O2
        cross_tile("fdf_cross_tile_large", data2, args.cross_tile_events, f2, g2)
        del data2
    # effect of the integral arithmetic on LL and gradient (GPU FdF, FP64 reductions)
    out["fdf_integral_variant"] = {}
    base = None
    for p in ["fp64"] + precs:
        L = R.pwaLikelihood()
        L.init(names, refl, None, RANK, 0.0)
        L.addNormIntegral(copy(ints[p]))
        L.addAccIntegral(copy(accs[p]))
        for k, n in enumerate(names):
            L.addAmplitude(n, data[k])
        L.finishInit()
        f, gg = L.FdF(par)
        if base is None:
            base = (f, gg)
        else:
            out["fdf_integral_variant"][p] = {"ll_rel": abs(f - base[0]) / abs(base[0]),
                                              "grad_normwise": float(np.max(np.abs(gg - base[1])) /
                                                                     np.max(np.abs(base[1])))}
    line = {"metric": "precision sweep (errors against FP64)", "workload": "compass88: 87 waves + flat, rank 2, "
            "%d data / %d MC events" % (args.n_data, args.n_mc), "data": "synthetic", "results": out}
    emit(line, args)
    return 0


def run_config0(args):
    """The single-bin configuration of the reference's own CPU-runnable case:
    15 positive-reflectivity waves + flat, rank 1, 20,000 data events,
    100,000 MC events with Bernoulli(0.6) acceptance, seed 0 (complex128
    amplitudes as drawn; the GPU stores them as complex64).  Timed on the GPU
    and, beside it, with the FP64 oracle on one host core (the reference's own
    threading): the normalisation + acceptance integral pair, one FdF, and one
    full fit from the same start point -- the GPU's L-BFGS to a gradient
    norm of 1e-6, scipy's L-BFGS-B on the oracle with the same tolerance
    (the reference's NLopt fit stops at xtol_rel 1e-4 / ftol_abs 1e-6,
    highLevelInterface/pwaNloptFit.cc:105-107, a looser criterion)."""
    import torch
    import scipy.optimize as so
    import rootpwa_gb300 as R
    from rootpwa_gb300 import synth
    from oracle.oracle import OracleIntegral, OracleLikelihood
    w = synth.make_workload("compass15", seed=0)
    names, refl = w["names"], w["refl"]
    mc128, data128 = w["mc"].astype(np.complex128), w["data"].astype(np.complex128)
    reps = max(3, min(args.steps, 20))

    def best(fn, n=reps):
        ts = []
        for _ in range(n):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return min(ts), statistics.median(ts)

    # ---- GPU: integral pair from host amplitudes, FdF, full fit ----
    def gpu_integrals():
        gn, ga = R.ampIntegralMatrix(), R.ampIntegralMatrix()
        gn.integrate(names, w["mc"], precision="tf32x3")
        ga.integrate(names, w["mc"], inBin=w["accepted"], precision="tf32x3")
        return gn, ga
    gpu_integrals()
    int_gpu, _ = best(gpu_integrals)
    gn, ga = gpu_integrals()
    snap = (integral_snapshot(gn), integral_snapshot(ga))
    L = R.pwaLikelihood()
    L.init(names, refl, None, 1, 0.0)
    L.addNormIntegral(gn)
    L.addAccIntegral(ga)
    for k, n in enumerate(names):
        L.addAmplitude(n, w["data"][k])
    L.finishInit()
    par = w["par"]
    for _ in range(5):
        L.FdF(par)
    fdf_gpu, fdf_gpu_med = best(lambda: L.FdF(par), n=200)
    M = R.pwaMultibin()
    M.setOptions(startGroup=8, gtolAbs=1e-6, gtolRel=0.0, maxIter=20000)
    M.addBin(L, 1)
    M.fit(par[None, :], sweepsPerGraph=20)
    torch.cuda.synchronize()
    fit_gpu_runs = []
    for _ in range(reps):
        t0 = time.perf_counter()
        res = M.fit(par[None, :], sweepsPerGraph=20)
        fit_gpu_runs.append(time.perf_counter() - t0)
    fit_gpu = statistics.median(fit_gpu_runs)

    # ---- CPU: the FP64 oracle, one thread ----
    def cpu_integrals():
        on, oa = OracleIntegral(), OracleIntegral()
        assert on.integrate(names, mc128) and oa.integrate(names, mc128, in_bin=w["accepted"])
        return on, oa
    int_cpu, _ = best(cpu_integrals, n=3)
    on, oa = cpu_integrals()
    O = OracleLikelihood()
    assert O.init(names, refl, None, 1, 0.0)
    assert O.addNormIntegral(on) and O.addAccIntegral(oa)
    for k, n in enumerate(names):
        assert O.addAmplitude(n, data128[k])
    assert O.finishInit()
    fdf_cpu, _ = best(lambda: O.FdF(par, threads=1), n=5)
    t0 = time.perf_counter()
    r = so.minimize(lambda p: O.FdF(p, threads=1), par, jac=True, method="L-BFGS-B",
                    options=dict(maxiter=20000, maxcor=8, gtol=1e-6, ftol=1e-15))
    fit_cpu = time.perf_counter() - t0
    # the GPU fit's minimum evaluated by the oracle with the GPU's own integrals
    Og = oracle_with_integrals(names, refl, w["data"], snap[0], snap[1], 1)
    f_gpu_at_min = Og.FdF(res["x"][0])[0]
    x_cpu = O.CorrectParamSigns(r.x)
    x_gpu = O.CorrectParamSigns(res["x"][0])
    cov = O.CovarianceMatrix(O.Hessian(x_cpu))
    sig = np.sqrt(np.maximum(np.diag(cov), 1e-300))
    line = {"metric": "single-bin configuration: one full fit, GPU wall time", "value": fit_gpu, "unit": "s",
            "higher_is_better": False, "n_gpus": 1, "impl": "gb300", "data": "synthetic",
            "config": {"workload": "compass15: 15 waves (+) + flat, rank 1, 20000 data / 100000 MC events, seed 0",
                       "parameters": len(par), "gtol": "gradient norm 1e-6 (both)"},
            "fit": {"gpu_s_median": fit_gpu, "gpu_runs_s": fit_gpu_runs, "gpu_iterations": int(res["iterations"][0]),
                    "gpu_status": int(res["status"][0]), "cpu_s": fit_cpu, "cpu_iterations": int(r.nit),
                    "cpu_fdf_evaluations": int(r.nfev), "speedup": fit_cpu / fit_gpu,
                    "ll_gpu": float(res["f"][0]), "ll_cpu": float(r.fun),
                    "ll_rel_diff": abs(float(res["f"][0]) - float(r.fun)) / abs(float(r.fun)),
                    "ll_gpu_point_by_oracle": float(f_gpu_at_min),
                    "v_diff_sigma_max": float(np.max(np.abs(x_gpu - x_cpu) / sig))},
            "fdf": {"gpu_host_call_us": fdf_gpu * 1e6, "gpu_host_call_median_us": fdf_gpu_med * 1e6,
                    "cpu_us": fdf_cpu * 1e6, "speedup": fdf_cpu / fdf_gpu},
            "integral_pair": {"gpu_s": int_gpu, "gpu_precision": "tf32x3, host complex64 amplitudes uploaded",
                              "cpu_s": int_cpu, "speedup": int_cpu / int_gpu},
            "cpu_baseline": {"value": fit_cpu, "unit": "s", "cores": 1, "kind": "port",
                             "sample": "the whole fit, scipy L-BFGS-B on the FP64 oracle FdF (one thread)"}}
    emit(line, args)
    return 0


def run_next(args):
    """Measurements of the rows after the FdF path: the GPU Hessian at the
    88-wave shapes (against the FP64 oracle's on a sample), loading a raw
    amplitude file with on-the-fly binning, and the selection alone."""
    import shutil
    import torch
    import rootpwa_gb300 as R
    from rootpwa_gb300 import synth
    from oracle.oracle import OracleIntegral, OracleLikelihood
    names, refl = synth.wave_names(N_NEG, N_POS)
    W = len(names)
    rng = np.random.Generator(np.random.PCG64(1))
    model = synth.AmplitudeModel(W, 8, rng)
    P = synth.n_pars(N_NEG, N_POS, RANK)
    par = rng.standard_normal(P)
    out = {}

    def host_best(fn, reps=3):
        fn()
        best = 1e30
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best

    # ---- Hessian (pwaLikelihood.cc:639-859) ----
    mc = model.draw(np.random.Generator(np.random.PCG64(2)), 100_000)
    oi = OracleIntegral()
    assert oi.integrate(names, mc.astype(np.complex128))

    def gpu_int():
        I = R.ampIntegralMatrix()
        I.setWaveNames(names)
        I.setMatrix(oi.raw())
        I.setNmbEvents(oi.nmb_events())
        return I

    def gpu_lik(d):
        L = R.pwaLikelihood()
        L.init(names, refl, None, RANK, 0.0)
        L.addNormIntegral(gpu_int())
        L.addAccIntegral(gpu_int())
        for k, n in enumerate(names):
            L.addAmplitude(n, d[k])
        L.finishInit()
        return L

    data = synth.draw_device(model, args.n_data, seed=11)
    L = gpu_lik(data)
    t_h = host_best(lambda: L.Hessian(par))
    n_sample = 20_000
    sample = data[:, :n_sample].cpu().numpy()
    O = OracleLikelihood()
    assert O.init(names, refl, None, RANK, 0.0)
    assert O.addNormIntegral(oi) and O.addAccIntegral(oi)
    for k, n in enumerate(names):
        assert O.addAmplitude(n, sample[k].astype(np.complex128))
    assert O.finishInit()
    t0 = time.perf_counter()
    H0 = O.Hessian(par)
    t_o = time.perf_counter() - t0
    Hs = gpu_lik(torch.from_numpy(sample).cuda()).Hessian(par)
    out["hessian"] = {
        "events": args.n_data, "parameters": P,
        "gpu_s": t_h,
        "oracle_single_thread_s_per_event": t_o / n_sample,
        "oracle_single_thread_s_extrapolated": t_o / n_sample * args.n_data,
        "max_rel_err_vs_oracle_on_%d_events" % n_sample: float(np.max(np.abs(Hs - H0)) / np.max(np.abs(H0))),
        "timing": "host-timed Hessian() call, best of 3 after one warm-up; oracle timed once on the sample",
    }
    del L
    torch.cuda.empty_cache()

    # ---- raw amplitude file + on-the-fly binning (pwaLikelihood.cc:1110-1288, :1391-1440) ----
    tmp = tempfile.mkdtemp(prefix="pwa_amp_")
    try:
        host = data.cpu().numpy()
        g = np.random.Generator(np.random.PCG64(3))
        mass = g.uniform(0.5, 2.5, args.n_data)
        tprime = g.exponential(0.3, args.n_data)
        path = os.path.join(tmp, "events.amp")
        R.writeAmplitudeFile(path, names, host, {"mass": mass, "tPrime": tprime})
        nbytes = os.path.getsize(path)
        bounds = {"mass": (1.0, 1.5), "tPrime": (0.1, 1.0)}

        def load():
            Lf = R.pwaLikelihood()
            Lf.init(names, refl, None, RANK, 0.0)
            Lf.addNormIntegral(gpu_int())
            Lf.addAccIntegral(gpu_int())
            Lf.loadAmplitudeFiles([path], bounds)
            Lf.finishInit()
            return Lf
        Lf = load()
        sel = Lf.otfSelected()
        keep = (mass >= 1.0) & (mass < 1.5) & (tprime >= 0.1) & (tprime < 1.0)
        assert sel == int(keep.sum())
        t_load = host_best(load)
        dcols = {"mass": torch.from_numpy(mass).cuda(), "tPrime": torch.from_numpy(tprime).cuda()}

        def select():
            Ls = R.pwaLikelihood()
            Ls.init(names, refl, None, RANK, 0.0)
            Ls.addNormIntegral(gpu_int())
            Ls.addAccIntegral(gpu_int())
            Ls.setOnTheFlyBinning(bounds, dcols)
        t_sel = host_best(select)
        out["amplitude_file"] = {
            "file_bytes": nbytes, "events": args.n_data, "selected": sel,
            "load_s": t_load, "load_GBps": nbytes / t_load / 1e9,
            "note": "file in the page cache (loaded once before timing); load = setup of a likelihood from the "
                    "file with the selection, finishInit included",
            "selection_s": t_sel,
            "selection_note": "likelihood init + both integrals + GPU selection over %d device-resident events "
                              "x 2 variables" % args.n_data,
        }
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    line = {"metric": "rows after the FdF path: Hessian, amplitude-file ingestion with on-the-fly binning",
            "workload": "compass88: 87 waves + flat, rank 2, %d events" % args.n_data, "data": "synthetic",
            "results": out}
    emit(line, args)
    return 0


def run_isobar(args):
    """Decay amplitudes of the 88-wave pi- pi+ pi- isobar set (three spinless
    final-state particles, helicity formalism) for --n-data events: events/s.
    value: momenta resident in HBM, one call of pwa_isobar_amplitudes per step
    on torch's stream, CUDA events around the timed steps; e2e: host momenta
    in, host amplitudes out through the Python API (both copies inside); the
    FP64 oracle on a bounded sample as the CPU baseline."""
    import ctypes as C
    import torch
    from rootpwa_gb300 import _native as Nn
    from rootpwa_gb300 import isobar as I
    from rootpwa_gb300 import synth
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    kws = synth.three_pion_waves()
    W, n = len(kws), args.n_data
    beam, fs, masses, mb = synth.three_pion_events(n, seed=31 + rank)
    A = I.isobarHelicityAmplitudes()
    A.setFinalState(["pi-", "pi+", "pi-"], masses, mb)
    for kw in kws:
        A.addWave(**kw)
    stream = torch.cuda.current_stream()
    A.setStream(stream)
    dev = torch.device("cuda", local)
    b = torch.from_numpy(np.ascontiguousarray(beam.T)).to(dev)                        # [3][N]
    f = torch.from_numpy(np.ascontiguousarray(np.transpose(fs, (0, 2, 1)))).to(dev)   # [3][3][N]
    outs = {"complex64": torch.empty((W, n), dtype=torch.complex64, device=dev),
            "complex128": torch.empty((W, n), dtype=torch.complex128, device=dev)}
    steps = max(1, min(args.steps, 50))

    def timed(dtype, clocked=False):
        out = outs[dtype]
        t = Nn.COMPLEX64 if dtype == "complex64" else Nn.COMPLEX128

        def step():
            Nn.call("pwa_isobar_amplitudes", A._h, C.c_void_p(b.data_ptr()), C.c_void_p(f.data_ptr()), n,
                    C.c_void_p(out.data_ptr()), t, Nn.MEMORY_DEVICE)
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        launches0 = Nn.lib().pwa_kernel_launch_count()
        clocks = ClockSampler(local) if clocked else None
        if clocks:
            clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        clk = clocks.stop() if clocks else None
        return e0.elapsed_time(e1) / steps, Nn.lib().pwa_kernel_launch_count() - launches0, clk

    ms, launches, clk = timed("complex64", clocked=True)
    ms64, _, _ = timed("complex128")
    # parity of the timed output on a sample against the FP64 oracle
    from oracle import isobar_oracle as O
    n_check = min(n, 1000)
    ows = [O.wave(kw["J"], kw["P"], kw["M"], kw["refl"], kw["L"], kw["S"], kw["isobarJ"], kw["isobarL"],
                  I.MASS_DEPENDENCES[kw["massDependence"]], kw["isobarMass"], kw["isobarWidth"],
                  kw["isobarDaughters"], kw["bachelor"]) for kw in kws]
    t0 = time.perf_counter()
    ref = O.amplitudes(ows, beam[:n_check], fs[:, :n_check], masses, mb, [0, 1, 0])
    t_cpu = time.perf_counter() - t0
    err = {}
    for dtype, o in outs.items():
        got = o[:, :n_check].cpu().numpy().astype(np.complex128)
        err[dtype] = max(float(np.abs(got[k] - ref[k]).max() / np.abs(ref[k]).max()) for k in range(W))
    # end to end through the Python API with host buffers
    B = I.isobarHelicityAmplitudes()
    B.setFinalState(["pi-", "pi+", "pi-"], masses, mb)
    for kw in kws:
        B.addWave(**kw)
    B.amplitudes(beam, fs, dtype="complex64")
    e2e_steps = max(1, min(steps, 5))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        B.amplitudes(beam, fs, dtype="complex64")
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    hbm, peak_kind = measured_peaks()
    algo_bytes = n * (12 * 8 + W * 8)
    achieved = algo_bytes / (ms * 1e-3) / 1e9
    line = {
        "metric": "isobar amplitudes: events/s at 88 waves (pi- pi+ pi-, helicity formalism)",
        "value": n / (ms * 1e-3), "unit": "events/s", "n_gpus": 1, "steps": steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 frames, f32 per-wave arithmetic, complex64 out",
        "fp64_mode": {"ms_per_step": ms64, "value": n / (ms64 * 1e-3), "unit": "events/s",
                      "dtype": "f64 throughout, complex128 out"},
        "data": "synthetic: seeded diffractive 3pi events (phase space), 88-wave isobar set",
        "config": {"workload": "isobar3pi88", "events": n, "waves": W, "sym_terms": A.nmbSymTerms(0),
                   "l2": "inputs and outputs (%.2f GB) larger than L2" % (algo_bytes / 1e9)},
        "e2e": {"value": n / t_e2e, "unit": "events/s", "h2d_bytes_per_step": n * 12 * 8,
                "d2h_bytes_per_step": n * W * 8},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": None, "peak_kind": peak_kind,
                     "note": ("algorithmic bytes (96 B in + 8 B per wave out per event, complex64 mode); the "
                              "kernel is not HBM-bound: it is latency-bound on the per-wave FP32 arithmetic "
                              "and its plan loads (ncu: issue active 49 %, DRAM < 1 %; "
                              "profiles/isobar_amplitude_kernel_3pi88.md)")},
        "cpu_baseline": {"value": n_check / t_cpu, "unit": "events/s", "cores": 1, "kind": "port",
                         "sample": "FP64 oracle (numpy) on %d events x %d waves" % (n_check, W)},
        "max_rel_err_vs_oracle": err,
        "timing": "CUDA events on torch's stream (pwa_isobar_set_stream), device-resident momenta",
        "clocks": clk,
    }
    emit(line, args)
    return 0


def main():
    args = parse()
    if args.workload == "precision":
        return run_precision(args)
    if args.workload == "next":
        return run_next(args)
    if args.workload == "isobar":
        return run_isobar(args)
    if args.workload == "config0":
        return run_config0(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "multibin":
        return run_multibin(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
