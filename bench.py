"""Benchmark: learned warm start + Richardson-Lucy light-field deconvolution on one GB300.

Default workload ("warmstart", the metric's configuration): Nnum 15, 30 x 30
lenslets (450 x 450 px), 21 z planes at -50..50 um, PSF generated on the GPU
for M40 / NA 0.95 / 150 um lenslets / f_ml 3000 um / 520 nm.  A 3-D U-Net is
trained on the GPU on synthetic bead + filament volumes (forward projected,
+100 background, Poisson noise); 256 held-out volumes decide how many RL
iterations after the network reach the data-fit residual of 8 plain-RL
iterations from a uniform volume.  One step = one deconvolved volume at that
accuracy: back projection Htf, the network's start volume, those RL
iterations.  ``value`` is that arm's volumes/s; the plain-RL arm (Htf, uniform
start, 8 Prevedel iterations), both arms' errors against the ground truth, the
roofline of the multiply-accumulate kernel, the FP32-vs-FP64 error (committed
FP64-oracle fixture) and the reference's own C++/FFTW CPU path on the same
geometry are reported in the same JSON line.

Other workloads (``--workload``): "small" (plain RL, 450 x 450, 11 planes),
"fullfield" (plain RL, 1005 x 1005, 41 planes), "timeseries" (mixed-size
frames), "psf", "rectify", "conv16" / "unet" (network kernels alone),
"warmstart_fullfield".

Prints one JSON line (rank 0).  ``--impl reference`` times the reference's own
C++/FFTW CPU path (Projector_allC + DeconvRL, built from the reference's
sources by oracle/ref_build.py) on the workload's geometry with all host cores.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "fast-light-field_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "volumes/s to plain-RL(8 it) accuracy: learned warm-start vs plain RL, 1 GB300"

# DRAM bytes (read + write) per k_mac launch over the bytes it streams, from one
# ncu --set full capture of the full-field f = 96 launches (4 planes, 1225
# frequency quads: 1.022 forward, 1.016 back projection).  The matrices dominate
# both, so the traffic of a launch scales with the bytes it streams.
MAC_TRAFFIC_RATIO = 1.02
UNIT = "volumes/s"

WORKLOADS = {
    # name: (Nnum, lenslets, z_min, z_max, z_step, psf size ref (lenslets at z_max), beads, filaments)
    "fullfield": dict(Nnum=15, lenslets=67, z=(-100, 100, 5), img_size_ref=28, beads=2000, filaments=50,
                      fp64_case="1005px_41planes",
                      label="full-field 1005x1005 px, Nnum 15, 41 planes -100..100 um, plain RL"),
    "small": dict(Nnum=15, lenslets=30, z=(-25, 25, 5), img_size_ref=7, beads=200, filaments=0,
                  fp64_case="450px_11planes",
                  label="450x450 px, Nnum 15, 11 planes -25..25 um, plain RL"),
    # GPU PSF generation for the optics of the 450 x 450 workload (M40 / NA 0.95 water, 150 um
    # lenslets, f_ml 3000 um, 520 nm, OSR 3)
    "psf": dict(Nnum=15, z=(-25, 25, 5), optics=dict(M=40, NA=0.95, MLPitch=150e-6, OSR=3, n=1.33, fml=3000e-6,
                                                     lam=520e-9),
                label="PSF generation, Nnum 15, M40 NA 0.95, OSR 3, 11 planes -25..25 um"),
    # learned warm start (450 x 450 px, Nnum 15, 21 planes at -50..50 um, PSF generated on the GPU for
    # the M40 / NA 0.95 optics); 200 beads per volume, background 100, Poisson noise
    # (img_size_ref 14: the PSF sizes, 61..421, the generator derives for these optics; the reference CPU
    # arm uses a synthetic set of those sizes)
    "warmstart": dict(Nnum=15, lenslets=30, z=(-50, 50, 5), beads=200, filaments=10, img_size_ref=14,
                      optics=dict(M=40, NA=0.95, MLPitch=150e-6, OSR=3, n=1.33, fml=3000e-6, lam=520e-9),
                      fp64_case="450px_21planes",
                      label="learned warm start + RL vs plain RL(8 it): 450x450 px (30x30 lenslets), Nnum 15, "
                            "21 planes -50..50 um, bead + filament volumes, 256 held-out seeds"),
    # the learned warm start on the full-field workload (synthetic PSF of the default workload)
    "warmstart_fullfield": dict(Nnum=15, lenslets=67, z=(-100, 100, 5), img_size_ref=28, beads=2000, filaments=50,
                                psf="synthetic",
                                label="learned warm start + RL vs plain RL(8 it), full field 1005x1005 px, Nnum 15, "
                                      "41 planes -100..100 um"),
    # Nnum 19, 101 x 101 lenslets, 51 planes at -125..125 um (125 um lenslets, f_ml 2500 um, M40, NA 0.95:
    # the reference's size rule gives PSFs of 41 lenslets at the deepest plane, sides up to 1559 px), 16 frames
    # per launch, 5000 beads + 200 filaments per volume; synthetic PSF set of those sizes
    "config4": dict(Nnum=19, lenslets=101, z=(-125, 125, 5), img_size_ref=41, beads=5000, filaments=200,
                    label="Nnum 19, 101x101 lenslets (1919x1919 px), 51 planes -125..125 um, 16 frames per launch, "
                          "plain RL(8 it), 5000 beads + 200 filaments"),
    # rectification of raw 2048 x 2048 16-bit camera images (lenslet period 14.73 px) to Nnum 15
    "rectify": dict(Nnum=15, raw=(2048, 2048), dx=14.73, label="rectify 2048x2048 uint16 raw images to Nnum 15"),
    # the warm-start network's kernels alone on a random BF16 volume (--shape Z Y X, default 24 456 456,
    # the padded 450 x 450 px x 21-plane volume): one 16 -> 16 channel 3x3x3 convolution, or the U-Net forward
    "conv16": dict(label="warm-start network: one 16->16 channel 3x3x3 BF16 convolution"),
    "unet": dict(label="warm-start network: U-Net forward (16-32-64-128 channels) with its head"),
    # a time series of frames of three sizes (--frames per size, default 32), 500 drifting beads each
    "timeseries": dict(Nnum=15, sizes=(30, 45, 67), z=(-75, 75, 5), img_size_ref=21, beads=500,
                       label="time series, Nnum 15, 31 planes -75..75 um, frames at 30x30, 45x45 and 67x67 "
                             "lenslets, RL from x0 = Htf"),
}


def set_mac_shape(ctx, spec):
    """--mac STAGES,ROWS_FWD,ROWS_BWD,SPLIT[,CTAS_PER_SM]: the multiply-accumulate launch shape (a sweep)."""
    if not spec:
        return
    v = [int(t) for t in spec.split(",")]
    ctx.set_option("mac_stages", v[0])
    ctx.set_option("mac_chunk_rows_forward", v[1])
    ctx.set_option("mac_chunk_rows_backward", v[2])
    ctx.set_option("mac_split", v[3])
    if len(v) > 4:
        ctx.set_option("mac_ctas_per_sm", v[4])


def pinned_empty(shape):
    """A float32 numpy array backed by page-locked host memory."""
    import torch
    return torch.empty(tuple(shape), dtype=torch.float32, pin_memory=True).numpy()


def pinned_like(a):
    """A page-locked host copy of a (numpy array or tensor) as a float32 numpy array."""
    import torch
    src = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a, np.float32)
    out = pinned_empty(src.shape)
    out[...] = src
    return out


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 200 for the warm-start workload, whose steps take ~1.5 ms, "
                         "so the clock sampler sees the timed region; 10 otherwise)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="warmstart", choices=sorted(WORKLOADS))
    ap.add_argument("--iters", type=int, default=8)
    ap.add_argument("--frames", type=int, default=1)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--train-steps", type=int, default=1600, help="warm-start network training steps")
    ap.add_argument("--held-out", type=int, default=0,
                    help="held-out volumes of the warm-start evaluation (0: 256 at 450 x 450, 16 at full field)")
    ap.add_argument("--target-iters", type=int, default=32,
                    help="plain-RL iterations the warm-start network learns to reach")
    ap.add_argument("--tune-steps", type=int, default=-1,
                    help="warm-start fine-tuning steps on the data-fit residual (whole volumes) after training "
                         "(default: 300 at 450 x 450, none at full field)")
    ap.add_argument("--streams", type=int, default=2, choices=[1, 2],
                    help="streams the transform groups alternate over (config4)")
    ap.add_argument("--no-graph", action="store_true", help="launch the RL kernels one by one instead of replaying a CUDA graph")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--shape", type=int, nargs=3, default=[24, 456, 456], metavar=("Z", "Y", "X"),
                    help="volume of the conv16 / unet network workloads")
    ap.add_argument("--kernel", default="tcgen05-all",
                    choices=["tcgen05", "tcgen05-all", "tcgen05-noswizzle", "mma.sync"],
                    help="conv16 / unet: tcgen05 = the 16->16 layers on tcgen05; tcgen05-all (the default) = "
                         "the 32-channel layers too")
    ap.add_argument("--wide", type=int, default=1, choices=range(6),
                    help="unet: kernel of the 64/128-channel layers (0 mma.sync, 1 tcgen05, 2..5 tcgen05 with "
                         "1..4 M tiles per work item)")
    ap.add_argument("--mac", default=None, metavar="STAGES,ROWS_FWD,ROWS_BWD,SPLIT[,CTAS_PER_SM]",
                    help="projection workloads: the multiply-accumulate launch shape (default: the library's)")
    ap.add_argument("--planes", default=None,
                    help="comma-separated z indices of the workload to keep (smaller cases for profiling)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 200 if args.workload == "warmstart" and args.impl == "gb300" else 10
    return args


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def build_problem(wl, seed=1234, keep=None):
    import psfmatrix
    import synthetic
    N = wl["Nnum"]
    z0, z1, dz = wl["z"]
    z = np.arange(z0, z1 + dz / 2, dz)
    if keep is not None:
        z = z[keep]
    H, Ht = synthetic.synthetic_psf(N, z, wl["img_size_ref"])
    hm = psfmatrix.HMatrixArrays(H, Ht, name="bench-%s" % wl["label"])
    Y = X = wl["lenslets"] * N
    gt, _ = synthetic.bead_volume((len(z), Y, X), wl["beads"], seed=seed, sigma=1.0,
                                  amp_range=(500.0, 1000.0))
    if wl["filaments"]:
        gt = gt + synthetic.filament_volume((len(z), Y, X), wl["filaments"], seed=seed + 1, width=1.5,
                                            intensity=500.0)
    return hm, H, Ht, z, gt.astype(np.float32), Y, X


class ClockSampler:
    """nvidia-smi samples (every 50 ms) of SM clock and throttle reasons.  A reader
    thread stamps each sample with the host time it arrives; mark() brackets the
    timed region, and stop() keeps the samples inside it (the first one after it
    when the region is shorter than the sampling interval)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def start(self):
        import threading
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return

        def reader():
            for line in self.proc.stdout:
                self.lines.append((time.time(), line))
        self.thread = threading.Thread(target=reader, daemon=True)
        self.thread.start()

    def mark(self, begin):
        if begin:
            self.t0 = time.time()
        else:
            self.t1 = time.time()

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=5)
        rows = self.lines
        if self.t0 is not None and self.t1 is not None:
            inside = [r for r in rows if self.t0 <= r[0] <= self.t1 + 0.06]
            after = [r for r in rows if r[0] >= self.t0]
            rows = inside if inside else after[:1]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, line in rows:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1", "0x1"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def survey_psf_bytes(N, Y, X, hs):
    """Compulsory PSF-spectrum bytes of one projection: sum over planes of
    K * F_z * (F_z / 2 + 1) * 8, K = n_h (n_h + 1) / 2 stored PSFs per plane,
    F_z = Nnum * ceil((max(Y, X) + h_z - 1) / Nnum) (the reference's GPU padding)."""
    nh = (N + 1) // 2
    K = nh * (nh + 1) // 2
    tot = 0
    for h in hs:
        F = N * (-(-(max(Y, X) + h - 1) // N))
        tot += K * F * (F // 2 + 1) * 8
    return float(tot)


def mac_roofline(prof, survey_bytes, what):
    """Roofline of k_mac from a per-kernel profile pass: achieved = the compulsory
    PSF-spectrum bytes of the projections profiled (survey_psf_bytes) over the
    kernel's total CUDA-event time, against the measured HBM copy peak; the
    kernel's own streamed bytes and their fraction beside it."""
    peak, peak_kind = measured_peaks()
    mac = {k: v for k, v in prof.items() if k.startswith("k_mac")}
    tot_ms = sum(v["ms"] for v in mac.values())
    own = sum(v["bytes"] for v in mac.values())
    n = max(1, sum(v["launches"] for v in mac.values()))
    ach = survey_bytes / (tot_ms / 1000.0) / 1e9 if tot_ms > 0 else 0.0
    own_ach = own / (tot_ms / 1000.0) / 1e9 if tot_ms > 0 else 0.0
    tot_all = sum(w["ms"] for w in prof.values()) or 1.0
    return {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 4),
            "traffic": round(own / n * MAC_TRAFFIC_RATIO),
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per k_mac launch, as a ratio to "
                              "the kernel's own streamed bytes (%.3f), times this run's own bytes per launch"
                              % MAC_TRAFFIC_RATIO,
            "kernel": "k_mac_fwd+k_mac_bwd", "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
            "launches": n, "avg_launch_ms": tot_ms / n,
            "algorithmic_bytes_per_launch": survey_bytes / n,
            "algorithmic_bytes": "sum over planes of K F_z (F_z/2+1) 8 B per projection, K = 36 stored PSFs, "
                                 "F_z = Nnum ceil((Y + h_z - 1) / Nnum); %s" % what,
            "own_bytes_per_launch": own / n, "own_achieved": round(own_ach, 1),
            "own_frac": round(own_ach / peak, 4),
            "kernel_share": {k: round(v["ms"] / tot_all, 4) for k, v in prof.items()}}


def reference_geometry(wl):
    """(Nnum, z planes, PSF sizes, Y, X) of a projection workload."""
    import synthetic
    N = wl["Nnum"]
    z0, z1, dz = wl["z"]
    z = np.arange(z0, z1 + dz / 2, dz)
    hs = synthetic.psf_sizes(N, z, wl["img_size_ref"])
    return N, z, hs, wl["lenslets"] * N, wl["lenslets"] * N


# Reference CPU arm: one step is one RL iteration (forward + back projection +
# update) where that takes seconds on the host, one back projection on the
# larger workloads.
REF_STEP = {"warmstart": "iteration", "small": "iteration", "fullfield": "projection",
            "warmstart_fullfield": "projection"}


def reference_line(workload, steps, warmup, iters, n_gpus):
    """Time the reference's own C++/FFTW CPU path (Projector_allC + DeconvRL, built
    from the reference's sources by oracle/ref_build.py) on the workload's geometry,
    with all host cores.  The PSF values are a synthetic set with the workload's PSF
    sizes (the work depends only on the shapes).  Falls back to the oracle's numpy
    restatement of the same algorithm ("port") when the reference cannot be built."""
    import shutil
    import tempfile
    import synthetic
    wl = WORKLOADS[workload]
    N, z, hs, Y, X = reference_geometry(wl)
    Z = len(z)
    cores = os.cpu_count() or 1
    H, Ht = synthetic.synthetic_psf(N, z, wl["img_size_ref"])
    img = synthetic.poisson_image(np.full((1, Y, X), 50.0, np.float32), 100.0, seed=3)
    kind, why = "reference", None
    try:
        from oracle import ref_build
        t0 = time.time()
        rprojector, rlfdeconv, rpsfmatrix, _ = ref_build.load()
        build_s = time.time() - t0
    except Exception as e:          # no C++ toolchain result: the numpy restatement
        kind, why, build_s = "port", "%s: %s" % (type(e).__name__, e), 0.0
    step_kind = REF_STEP[workload]
    cwd = os.getcwd()
    tmp = tempfile.mkdtemp(prefix="flf_ref_")
    os.chdir(tmp)       # the reference writes overall.txt / mutex_report_static.txt into the working directory
    noprog = lambda w, desc=None, leave=True, **k: w   # noqa: E731
    try:
        if kind == "reference":
            shapes = []
            for zi, (h, ht) in enumerate(zip(H, Ht)):
                for nm, arr in (("H", h), ("Ht", ht)):
                    m = np.memmap(os.path.join(tmp, "%s%02d.array" % (nm, zi)), dtype="float32", mode="w+",
                                  shape=arr.shape)
                    m[...] = arr
                    m.flush()
                    del m
                shapes.append(h.shape)
            hm = rpsfmatrix.HMatrix(os.path.join(tmp, "H{z:02d}.array"), os.path.join(tmp, "Ht{z:02d}.array"), shapes)
            proj = rprojector.Projector_allC()

            def backward():
                return proj.BackwardProjectACC(hm, img, range(Z), noprog, False, cores)

            def iteration(htf, x):
                return rlfdeconv.DeconvRL(hm, htf, 1, x, logPrint=False, numjobs=cores, projector=proj,
                                          progress=noprog)
            impl = "reference C++/FFTW path (Projector_allC, DeconvRL), built from the reference's sources"
        else:
            from oracle import lf_oracle as O

            def backward():
                return np.stack([O.project_plane_ref_cpu(img, Ht[zi], N, workers=cores) for zi in range(Z)])

            def iteration(htf, x):
                hx = sum(O.project_plane_ref_cpu(x[zi], H[zi], N, workers=cores) for zi in range(Z))
                bp = np.stack([O.project_plane_ref_cpu(hx, Ht[zi], N, workers=cores) for zi in range(Z)])
                with np.errstate(divide="ignore", invalid="ignore"):
                    x = x * (htf / bp)
                x[np.isnan(x)] = 0
                return x
            impl = "oracle numpy restatement of the reference's CPU algorithm (%s)" % why
        t0 = time.time()
        htf = backward()                     # first call: FFTW planning, memmaps paged in
        first_s = time.time() - t0
        t0 = time.time()
        htf = backward()
        t_bwd = time.time() - t0
        x = np.ones_like(htf)
        times = []
        for i in range(warmup + steps):
            t0 = time.time()
            if step_kind == "iteration":
                x = iteration(htf, x)
            else:
                backward()
            if i >= warmup:
                times.append(time.time() - t0)
    finally:
        os.chdir(cwd)
        shutil.rmtree(tmp, ignore_errors=True)
    t_step = float(np.mean(times))
    if step_kind == "iteration":
        vol_s = t_bwd + iters * t_step
        sample = ("%d timed RL iterations (each a forward and a back projection of all %d planes and the update) "
                  "after %d warm-up iterations; one volume = back projection %.2f s + %d iterations" %
                  (steps, Z, warmup, t_bwd, iters))
    else:
        vol_s = (1 + 2 * iters) * t_step
        sample = ("%d timed back projections of all %d planes after %d warm-up; one volume = %d projections "
                  "(a forward projection streams the same spectra)" % (steps, Z, warmup, 1 + 2 * iters))
    return {"impl": "reference", "metric": METRIC if workload == "warmstart" else
            "volumes/s to plain-RL(8 it) accuracy, CPU", "value": 1.0 / vol_s, "unit": UNIT,
            "n_gpus": n_gpus, "steps": steps, "warmup": warmup, "ms_per_step": t_step * 1000.0,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": wl["label"], "image": [Y, X], "planes": Z, "nnum": N, "psf_sizes": hs,
                       "rl_iterations": iters, "frames": 1, "implementation": impl,
                       "step": step_kind, "first_call_s": round(first_s, 2), "build_or_load_s": round(build_s, 1)},
            "rl_iterations_per_s": iters / vol_s,
            "cpu_baseline": {"value": 1.0 / vol_s, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample,
                             "seconds_per_volume": vol_s},
            "e2e": {"value": 1.0 / vol_s, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def cpu_baseline_subprocess(workload, iters, steps=2, warmup=1, timeout=900):
    """The reference CPU arm on a bounded sample, in a separate process (the
    reference's modules share names with this package's); None if it fails."""
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--workload", workload,
           "--steps", str(steps), "--warmup", str(warmup), "--iters", str(iters)]
    try:
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=timeout,
                           cwd=ROOT)
        line = json.loads(r.stdout.strip().splitlines()[-1])
        cb = dict(line["cpu_baseline"])
        cb["implementation"] = line["config"]["implementation"]
        return cb
    except Exception as e:
        return {"value": None, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": None,
                "sample": "reference CPU arm failed: %s" % (str(e)[:200])}


def run_reference(args, rank, world):
    if rank != 0:
        return
    if args.workload not in REF_STEP:
        print(json.dumps({"impl": "reference", "unavailable": "the CPU reference arm is timed on the projection "
                          "workloads; this workload reports its CPU oracle inside the GB300 line"}), flush=True)
        return
    print(json.dumps(reference_line(args.workload, args.steps, args.warmup, args.iters, args.gpus)), flush=True)


def run_gb300(args, rank, world, local):
    import torch
    import lfdeconv
    import projector
    import _flf
    import build_lib
    build_lib.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    wl = WORKLOADS[args.workload]
    N = wl["Nnum"]
    T = args.frames
    t_setup = time.time()
    keep = [int(v) for v in args.planes.split(",")] if args.planes else None
    hm, H, Ht, z, gt, Y, X = build_problem(wl, seed=1234 + rank, keep=keep)
    Z = len(z)
    p = projector.Projector_gb300(device=local)
    p.storeVolumesOnGPU = True
    gt_d = torch.as_tensor(gt[:, None], device=dev).repeat(1, T, 1, 1).contiguous()
    clean = p.ForwardProjectACC(hm, gt_d, None)
    gen = torch.Generator(device="cpu").manual_seed(99 + rank)
    img_h = torch.poisson((clean.cpu().double() + 100.0).clamp_min(0), generator=gen).float().numpy()
    ctx = p.context(hm)
    set_mac_shape(ctx, args.mac)
    geo = ctx.geometry()
    setup_s = time.time() - t_setup
    stream = torch.cuda.current_stream(dev)
    img_d = torch.as_tensor(img_h, device=dev)
    htf = torch.empty((Z, T, Y, X), dtype=torch.float32, device=dev)
    x = torch.empty((Z, T, Y, X), dtype=torch.float32, device=dev)

    # the RL iterations of a step replay one CUDA graph (flf_rl_graph_create)
    graph = None if args.no_graph else ctx.rl_graph(x, htf, None, _flf.FLF_RL_PREVEDEL, args.iters, T, Y, X)

    def step(direct=False):
        ctx.backward(img_d, htf, T, Y, X, None, stream=stream.cuda_stream)
        x.fill_(1.0)
        if graph is None or direct:
            ctx.rl_iterate(x, htf, None, _flf.FLF_RL_PREVEDEL, args.iters, T, Y, X, stream=stream.cuda_stream)
        else:
            graph.launch(stream.cuda_stream)

    def timed(direct):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            step(direct)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    clocks.mark(True)
    ms = timed(direct=False)
    clocks.mark(False)
    clk = clocks.stop()
    # per-kernel durations: the same steps again, launched directly on one
    # stream with CUDA events around every kernel (a graph replay has no
    # per-kernel events, and with two streams an event pair would also time the
    # other stream's kernels running beside it)
    ctx.set_option("streams", 1)
    ctx.profile(True)
    ms_direct = timed(direct=True)
    prof = ctx.profile_read()
    ctx.profile(False)
    ctx.set_option("streams", 2)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * T / (ms / 1000.0)

    # end to end through the public API: host image and start volume in, host volume out
    e2e = None
    if not args.no_e2e:
        p.storeVolumesOnGPU = False
        img_p = pinned_like(img_h)
        x0_h = pinned_empty((Z, T, Y, X))
        x0_h[...] = 1.0
        r = pinned_empty((Z, T, Y, X))
        lfdeconv.DeconvRL(hm, None, args.iters, x0_h, logPrint=False, projector=p, im=img_p, out=r)
        torch.cuda.synchronize()
        ne = max(1, min(args.steps, 5))
        t0 = time.perf_counter()
        for _ in range(ne):
            lfdeconv.DeconvRL(hm, None, args.iters, x0_h, logPrint=False, projector=p, im=img_p, out=r)
        e2e_s = (time.perf_counter() - t0) / ne
        e2e = {"value": world * T / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(img_h.nbytes + x0_h.nbytes),
               "d2h_bytes_per_step": int(r.nbytes), "ms_per_step": e2e_s * 1000.0}

    # roofline of the dominant kernel (the spectral multiply-accumulate)
    hs = [int(hm.PSFShape(c)[-1]) for c in range(Z)]
    roof = mac_roofline(prof, survey_psf_bytes(N, Y, X, hs) * args.steps * (1 + 2 * args.iters),
                        "%s, %d projections per step" % (wl["label"], 1 + 2 * args.iters))
    launches = sum(v["launches"] for v in prof.values()) // args.steps

    # accuracy of the volume the timed step produced (outside the timed region):
    # relative data-fit residual ||y - Hx|| / ||y|| and error against the
    # ground-truth volume, reduced in FP64
    hx = torch.empty((T, Y, X), dtype=torch.float32, device=dev)
    ctx.forward(x, hx, T, Y, X, None, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    y64 = img_d.double()
    resid = float(torch.linalg.vector_norm(y64 - hx.double()) / torch.linalg.vector_norm(y64))
    x64 = x.double()
    g64 = gt_d.double()
    scale = float((x64 * g64).sum() / (x64 * x64).sum())     # RL recovers the volume up to the PSF's scale
    accuracy = {"rl_iterations": args.iters, "residual_rel_l2": resid,
                "truth_rel_l2": float(torch.linalg.vector_norm(x64 - g64) / torch.linalg.vector_norm(g64)),
                "truth_rel_l2_scaled": float(torch.linalg.vector_norm(scale * x64 - g64) / torch.linalg.vector_norm(g64)),
                "reductions": "f64"}
    del hx, y64, x64, g64
    if wl.get("fp64_case") and keep is None:
        accuracy["fp64"] = fp64_accuracy(wl["fp64_case"], local)

    cb = None
    if rank == 0 and not args.no_cpu_baseline:
        cb = cpu_baseline_subprocess(args.workload, args.iters)

    if rank == 0:
        gb = ctx.memory_usage() / 1e9
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": wl["label"] + (" (planes %s only)" % args.planes if keep else ""),
                           "image": [Y, X], "planes": Z, "nnum": N, "frames": T,
                           "rl_iterations": args.iters, "rl_variant": "prevedel", "start": "uniform",
                           "projections_per_step": 1 + 2 * args.iters,
                           "transform_size": geo["f"], "kernel_radius_lenslets": geo["R"],
                           "precompute_fp64": geo["fp64"], "device_gb": round(gb, 2),
                           "setup_s": round(setup_s, 1),
                           "l2": "inputs larger than L2: %.1f GB of transfer matrices streamed per "
                                 "projection, %.0f MB volume" % (roof["own_bytes_per_launch"] * roof["launches"]
                                                                / args.steps / (1 + 2 * args.iters) / 1e9,
                                                                Z * T * Y * X * 4 / 1e6),
                           "parallelism": "replicas" if world > 1 else "single",
                           "rl_launch": "direct" if graph is None else
                           "CUDA graph replay of the RL iterations (%d kernels)" % graph.kernels},
                "ms_per_step_direct_profiled": ms_direct,
                "rl_iterations_per_s": value * args.iters, "accuracy": accuracy,
                "e2e": e2e, "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cb,
                "clocks": clk}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_timeseries(args):
    """Mixed-size time series on one device (32 frames of each size by
    default): per size, T frames back projected and deconvolved together (x0 = Htf,
    as the time-series driver does), the multiply-accumulate launch shape autotuned
    per size; each size's whole deconvolution (back projection, x0 = Htf, RL
    iterations) is captured as a graph and the three are combined into one graph,
    so one step (every frame of every size) is one graph launch.  The geometries of
    all sizes stay resident.  With T frames per launch the multiply-accumulate is
    FP32-bound: its roofline is reported against the nominal FP32 rate."""
    import torch
    import projector
    import psfmatrix
    import synthetic
    import warmstart
    import _flf
    import build_lib
    build_lib.build()
    dev = torch.device("cuda", 0)
    wl = WORKLOADS["timeseries"]
    N = wl["Nnum"]
    T = args.frames if args.frames > 1 else 32
    z0, z1, dz = wl["z"]
    z = np.arange(z0, z1 + dz / 2, dz)
    Z = len(z)
    H, Ht = synthetic.synthetic_psf(N, z, wl["img_size_ref"])
    hm = psfmatrix.HMatrixArrays(H, Ht, name="bench-timeseries")
    p = projector.Projector_gb300(device=0)
    p.storeVolumesOnGPU = True
    ctx = p.context(hm)
    ctx.set_option("geometry_cache", len(wl["sizes"]))
    rng = np.random.default_rng(4321)
    s = torch.cuda.current_stream(dev)
    data = []
    t_setup = time.time()
    for L in wl["sizes"]:
        Y = X = L * N
        # drifting beads rendered on the device: positions move N(0, 0.5 voxel) per frame
        pos = np.stack([rng.uniform(0, Z - 1, wl["beads"]), rng.uniform(0, Y - 1, wl["beads"]),
                        rng.uniform(0, X - 1, wl["beads"])], axis=1)
        amp = rng.uniform(500.0, 1000.0, wl["beads"])
        gt = torch.zeros((T, Z, Y, X), device=dev)
        acc = torch.empty(Z * Y * X, dtype=torch.int64, device=dev)
        for t in range(T):
            if t:
                pos = pos + rng.normal(0.0, 0.5, pos.shape)
            pts = torch.as_tensor(np.concatenate([pos, amp[:, None]], axis=1).astype(np.float32), device=dev)
            _flf.render_blobs(gt[t], pts, 1.0, s.cuda_stream, acc=acc)
        gt = gt.permute(1, 0, 2, 3).contiguous()
        clean = p.ForwardProjectACC(hm, gt, None)
        img = torch.poisson((clean.double() + 100.0).clamp_min(0)).float()
        data.append((Y, X, img))
        del gt, clean
    bufs = [(torch.empty((Z, T, Y, X), device=dev), torch.empty((Z, T, Y, X), device=dev)) for Y, X, _ in data]
    tuned = {}
    for (Y, X, _), _b in zip(data, bufs):
        tuned["%dx%d" % (Y, X)] = p.autotune(hm, T, Y, X)
    # one direct pass sizes every workspace before the graphs bake their addresses in
    for (Y, X, img), (htf, x) in zip(data, bufs):
        p._prepare(ctx, Y, X, hm)
        ctx.backward(img, htf, T, Y, X, None, stream=s.cuda_stream)
        x.copy_(htf)
        ctx.rl_iterate(x, htf, None, _flf.FLF_RL_PREVEDEL, args.iters, T, Y, X, stream=s.cuda_stream)
    torch.cuda.synchronize()
    graphs = []
    for (Y, X, img), (htf, x) in zip(data, bufs):
        p._prepare(ctx, Y, X, hm)
        graphs.append(ctx.deconv_graph(img, htf, x, args.iters, T, Y, X))
    whole = ctx.combine_graphs(graphs)
    setup_s = time.time() - t_setup

    def step():
        whole.launch(s.cuda_stream)

    for _ in range(max(args.warmup, 1)):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    clocks.mark(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(args.steps):
        step()
    e1.record(s)
    torch.cuda.synchronize()
    clocks.mark(False)
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    nvol = T * len(data)
    # per-kernel times: the same work launched directly between CUDA events on one
    # stream; FP32 roofline of the multiply-accumulate from the reference's count of
    # 8 N^2 F_z (F_z / 2 + 1) flops per plane, frame and projection
    hs = [int(hm.PSFShape(c)[-1]) for c in range(Z)]
    ctx.set_option("streams", 1)
    ctx.profile(True)
    flops = 0.0
    for (Y, X, img), (htf, x) in zip(data, bufs):
        p._prepare(ctx, Y, X, hm)
        ctx.backward(img, htf, T, Y, X, None, stream=s.cuda_stream)
        x.copy_(htf)
        ctx.rl_iterate(x, htf, None, _flf.FLF_RL_PREVEDEL, args.iters, T, Y, X, stream=s.cuda_stream)
        for h in hs:
            F = N * (-(-(max(Y, X) + h - 1) // N))
            flops += (1 + 2 * args.iters) * T * 8.0 * N * N * F * (F // 2 + 1)
    torch.cuda.synchronize()
    prof = ctx.profile_read()
    ctx.profile(False)
    ctx.set_option("streams", 2)
    mac = {k: v for k, v in prof.items() if k.startswith("k_mac")}
    mac_ms = sum(v["ms"] for v in mac.values())
    n_mac = max(1, sum(v["launches"] for v in mac.values()))
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
    tot = sum(v["ms"] for v in prof.values()) or 1.0
    roof = {"bound": "fp32", "kernel": "k_mac_fwd+k_mac_bwd", "unit": "TFLOP/s",
            "achieved": round(flops / (mac_ms / 1000.0) / 1e12, 2), "peak": round(fp32_peak, 1),
            "peak_source": "nominal FP32 FMA rate (152 SMs x 128 lanes x 2 flop x 2.07 GHz); MEASURED_PEAKS.json "
                           "has no FP32 figure",
            "frac": round(flops / (mac_ms / 1000.0) / 1e12 / fp32_peak, 4), "launches": n_mac,
            "avg_launch_ms": mac_ms / n_mac, "flops_per_launch": flops / n_mac,
            "kernel_share": {k: round(v["ms"] / tot, 4) for k, v in prof.items()}}
    line = {"metric": "volumes/s, mixed-size time series (8 plain-RL iterations from x0 = Htf), 1 GB300",
            "value": nvol / (ms / 1000.0), "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": wl["label"], "frames_per_size": T, "sizes_px": [Y for Y, _, _ in data],
                       "planes": Z, "nnum": N, "rl_iterations": args.iters, "volumes_per_step": nvol,
                       "rl_launch": "one CUDA graph for all sizes (%d kernels: back projection, x0 = Htf and "
                                    "the RL iterations of each size)" % whole.kernels,
                       "autotuned": tuned, "device_gb": round(ctx.memory_usage() / 1e9, 2),
                       "setup_s": round(setup_s, 1),
                       "l2": "inputs larger than L2 (transfer matrices of three geometries)"},
            "rl_iterations_per_s": nvol * args.iters / (ms / 1000.0), "roofline": roof,
            "gpu_launches": int(whole.kernels), "clocks": clk}
    print(json.dumps(line), flush=True)
    whole.close()
    for g in graphs:
        g.close()


def run_rectify(args):
    """Rectification throughput (images/s): the device resample alone (value) and the
    public RectifyImage call with host image in and host result out (e2e), beside the
    CPU oracle of the reference's RectifyImage on one image."""
    import torch
    import build_lib
    import rectify
    import _flf
    from oracle import rectify_oracle as R
    build_lib.build()
    wl = WORKLOADS["rectify"]
    T = max(args.frames, 8)
    H, W = wl["raw"]
    rng = np.random.default_rng(5)
    imgs = (rng.random((T, H, W)) * 60000).astype(np.uint16)
    kw = dict(xCenter_m=W / 2 + 0.37, yCenter_m=H / 2 - 0.21, dx=wl["dx"], Nnum=wl["Nnum"], Crop=False,
              XcutLeft=0, XcutRight=0, YcutUp=0, YcutDown=0)
    yq, xq, ny, nx = rectify.rectify_grid((H, W), kw["xCenter_m"], kw["yCenter_m"], kw["dx"], kw["Nnum"])
    dev = torch.device("cuda", 0)
    s = torch.cuda.current_stream(dev)
    img_d = torch.as_tensor(imgs.astype(np.float32), device=dev)
    yq_d = torch.as_tensor(np.ascontiguousarray(yq[:ny]), device=dev)
    xq_d = torch.as_tensor(np.ascontiguousarray(xq[:nx]), device=dev)
    out = torch.empty((T, ny, nx), dtype=torch.float64, device=dev)

    def step():
        for t in range(T):
            _flf.resample_bilinear(img_d[t], yq_d, xq_d, out[t], s.cuda_stream)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(args.steps):
        step()
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    rectify.RectifyImage(imgs[0], **kw)
    t0 = time.perf_counter()
    for t in range(T):
        rectify.RectifyImage(imgs[t], **kw)
    e2e_s = (time.perf_counter() - t0) / T
    t0 = time.perf_counter()
    R.rectify_image(imgs[0], **kw)
    cpu_s = time.perf_counter() - t0
    bytes_per_image = 4.0 * H * W + 8.0 * ny * nx
    line = {"metric": "raw light-field images/s rectified (bilinear resample), 1 GB300", "value": T / (ms / 1000.0),
            "unit": "images/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl["label"], "images_per_step": T, "out_px": [int(ny), int(nx)],
                       "l2": "inputs 16 MB per image, %d images per step" % T},
            "e2e": {"value": 1.0 / e2e_s, "unit": "images/s", "h2d_bytes_per_step": int(imgs[0].size * 4),
                    "d2h_bytes_per_step": int(8 * ny * nx)},
            "roofline": {"bound": "hbm", "achieved": round(bytes_per_image * T / (ms / 1000.0) / 1e9, 1),
                         "peak": measured_peaks()[0], "unit": "GB/s",
                         "frac": round(bytes_per_image * T / (ms / 1000.0) / 1e9 / measured_peaks()[0], 4)},
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "images/s", "cores": 1, "kind": "port",
                             "sample": "one image through the oracle restatement of RectifyImage (numpy)"}}
    print(json.dumps(line), flush=True)


def run_psf(args):
    """PSF generation (planes/s): GeneratePSFArrays on the device (value) and GeneratePSF
    writing the memmap files (e2e), beside the CPU oracle of the reference's generator on
    a 3-plane sample of the same optics."""
    import tempfile
    import warnings
    import torch
    import build_lib
    import generate_psf
    from oracle import psf_oracle as P
    build_lib.build()
    warnings.simplefilter("ignore")
    wl = WORKLOADS["psf"]
    z0, z1, dz = wl["z"]
    kw = dict(Nnum=wl["Nnum"], zmin=z0 * 1e-6, zmax=z1 * 1e-6, zspacing=dz * 1e-6, **wl["optics"])
    Z = len(np.arange(z0, z1 + dz / 2, dz))
    for _ in range(max(args.warmup, 3)):
        r = generate_psf.GeneratePSFArrays(**kw)
    torch.cuda.synchronize()
    steps = max(1, args.steps)
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    clocks.mark(True)
    t0 = time.perf_counter()
    tim = []
    for _ in range(steps):
        r = generate_psf.GeneratePSFArrays(**kw)
        tim.append(r["timings"])
    torch.cuda.synchronize()
    sec = (time.perf_counter() - t0) / steps
    clocks.mark(False)
    clk = clocks.stop()
    with tempfile.TemporaryDirectory() as d:
        t0 = time.perf_counter()
        generate_psf.GeneratePSF(matrixSaveDir=d, **kw)
        e2e_s = time.perf_counter() - t0
        nbytes = sum(os.path.getsize(os.path.join(dp, f)) for dp, _, fs in os.walk(d) for f in fs)
    sample = dict(kw, zspacing=(z1 - z0) / 2 * 1e-6)
    t0 = time.perf_counter()
    P.generate_psf(sample)
    cpu_s = time.perf_counter() - t0
    mean = {k: float(np.mean([t[k] for t in tim])) for k in tim[0]}
    line = {"metric": "PSF planes/s generated (Debye integral, microlens Fresnel propagation, binning, Ht), 1 GB300",
            "value": Z / sec, "unit": "planes/s", "n_gpus": 1, "steps": steps, "warmup": max(args.warmup, 3),
            "ms_per_step": sec * 1000.0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl["label"], "planes": Z, "image_grid": r["image_size"],
                       "psf_sizes": [int(h.shape[-1]) for h in r["H"]], "quadrature_nodes": mean["quadrature_nodes"],
                       "l2": "per plane 64 fields of %d x %d complex128 (%.0f MB)" % (
                           r["image_size"], r["image_size"], 64 * 16 * r["image_size"] ** 2 / 1e6)},
            "phases_s": {k: round(v, 4) for k, v in mean.items() if k.endswith("_s")},
            "e2e": {"value": Z / e2e_s, "unit": "planes/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": int(nbytes)},
            "roofline": {"bound": "fp64", "kernel": "k_psf_debye + cuFFT Z2Z (FP64 arithmetic)",
                         "achieved": None, "peak": None, "unit": None, "frac": None,
                         "note": "FP64-arithmetic bound; MEASURED_PEAKS has no FP64 figure"},
            "cpu_baseline": {"value": 3 / cpu_s, "unit": "planes/s", "cores": os.cpu_count() or 1, "kind": "port",
                             "sample": "oracle restatement of the reference's GeneratePSF (scipy quad_vec, numpy "
                                       "FFTs) on 3 of the 11 planes (z = %g, %g, %g um: the two largest and the "
                                       "smallest), %.1f s" % (z0, (z0 + z1) / 2, z1, cpu_s)},
            "clocks": clk}
    print(json.dumps(line), flush=True)


def fp64_accuracy(case, p_dev=0):
    """FP32 GPU Htf and Prevedel RL against the committed FP64-oracle fixture of a
    case (tests/golden/fp64_<case>.npz; same inputs regenerated from
    tests/golden/fp64_inputs.py): largest sampled error over the FP64 maximum and
    sampled relative L2 error.  None when the fixture is absent."""
    import torch
    import _flf
    import psfmatrix
    import projector
    gold = os.path.join(ROOT, "tests", "golden")
    if not os.path.exists(os.path.join(gold, "fp64_%s.npz" % case)):
        return None
    if gold not in sys.path:
        sys.path.insert(0, gold)
    import fp64_inputs as F
    c = F.CASES[case]
    H, Ht = F.psf(case)
    p = projector.Projector_gb300(device=p_dev)
    ctx = p.context(psfmatrix.HMatrixArrays(H, Ht))
    Z, Y, X = len(H), c["Y"], c["X"]
    dev = torch.device("cuda", p_dev)
    img = torch.as_tensor(F.image(case), device=dev)
    htf = torch.empty((Z, 1, Y, X), device=dev)
    s = torch.cuda.current_stream(dev).cuda_stream
    ctx.backward(img, htf, 1, Y, X, None, stream=s)
    x = torch.ones_like(htf)
    ctx.rl_iterate(x, htf, None, _flf.FLF_RL_PREVEDEL, c["iters"], 1, Y, X, stream=s)
    ctx.synchronize(s)
    e = F.compare(case, htf[:, 0].cpu().numpy(), x[:, 0].cpu().numpy())
    ctx.close()
    del p, htf, x
    torch.cuda.empty_cache()
    e.update({"case": case, "rl_iterations": int(c["iters"]), "checked_planes": F.checked_planes(case),
              "samples": F.SAMPLES, "psf": "synthetic set with the configuration's PSF sizes",
              "oracle": "float64 restatement of the reference's CPU algorithm (tests/golden/make_fp64_fixtures.py)"})
    return e


def run_warmstart(args):
    """Volumes/s to the data-fit residual of 8 plain-RL iterations: plain RL from a
    uniform volume against the learned warm start plus as many RL iterations as the
    held-out volumes need (the largest over them).  ``value`` is the warm-start arm;
    the plain-RL arm, both arms' errors against the ground-truth volumes, the k_mac
    roofline, the network convolution's tensor roofline, the FP32-vs-FP64 error and
    the reference's CPU path are reported beside it."""
    import warnings
    import torch
    import build_lib
    import generate_psf
    import psfmatrix
    import projector
    import warmstart
    import _flf
    build_lib.build()
    warnings.simplefilter("ignore")
    wl = WORKLOADS[args.workload]
    z0, z1, dz = wl["z"]
    # the reference's CPU path first, in its own process, before this one holds the GPU busy
    cb = None if args.no_cpu_baseline else cpu_baseline_subprocess(args.workload, 8)
    t0 = time.time()
    if wl.get("psf") == "synthetic":
        hm = build_problem(wl)[0]
        psf_desc = "synthetic (the default workload's), sizes %s" % [int(hm.PSFShape(c)[-1]) for c in range(hm.numZ)]
    else:
        r = generate_psf.GeneratePSFArrays(Nnum=wl["Nnum"], zmin=z0 * 1e-6, zmax=z1 * 1e-6, zspacing=dz * 1e-6,
                                           **wl["optics"])
        hm = psfmatrix.HMatrixArrays(r["H"], r["Ht"], name="bench-warmstart")
        psf_desc = "generated on the GPU (generate_psf.py), sizes %s" % [int(h.shape[-1]) for h in r["H"]]
    psf_s = time.time() - t0
    N = wl["Nnum"]
    Y = X = wl["lenslets"] * N
    Z = hm.numZ
    hs = [int(hm.PSFShape(c)[-1]) for c in range(Z)]
    p = projector.Projector_gb300()
    ws = warmstart.WarmStart(p, hm, Y, X, beads=wl["beads"], filaments=wl.get("filaments", 0))
    refresh = 8 if Y * X * Z < 10_000_000 else 16
    train_s = ws.train(steps=args.train_steps, batch=4, crop=128, target_iters=args.target_iters, log_every=1,
                       refresh_every=refresh)
    if args.tune_steps < 0:
        args.tune_steps = 300 if args.workload == "warmstart" else 0
    tune_s = ws.finetune_residual(steps=args.tune_steps, log_every=50) if args.tune_steps > 0 else 0.0
    dev = ws.dev
    s = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(2024)
    nseed = args.held_out if args.held_out > 0 else (256 if Y * X * Z < 10_000_000 else 16)
    ctx = ws.ctx
    set_mac_shape(ctx, args.mac)

    def resid(x, img):
        T = img.shape[0]
        hx = torch.empty_like(img)
        ctx.forward(x, hx, T, Y, X, None, stream=s.cuda_stream)
        d = (img.double() - hx.double()).reshape(T, -1)
        return (d.norm(dim=1) / img.double().reshape(T, -1).norm(dim=1)).cpu().numpy()

    def truth_err(x, truth):
        """Relative L2 error against the ground-truth volume after the best scale
        (RL recovers a volume up to the PSF's normalisation), per frame."""
        xs = x.double().permute(1, 0, 2, 3).reshape(x.shape[1], -1)
        g = truth.double().permute(1, 0, 2, 3).reshape(truth.shape[1], -1)
        a = (xs * g).sum(dim=1) / (xs * xs).sum(dim=1).clamp_min(1e-300)
        return ((a[:, None] * xs - g).norm(dim=1) / g.norm(dim=1)).cpu().numpy()

    # held-out volumes in chunks that keep the network's activations small
    chunk = max(1, min(nseed, 40_000_000 // (Z * Y * X)))
    r_plain, t_plain, curves, tcurves, need = [], [], [], [], []
    for c0 in range(0, nseed, chunk):
        truth, imgs, htfs = ws.make_batch(min(chunk, nseed - c0), rng)
        xu = torch.ones_like(htfs)
        p.RichardsonLucy(hm, xu, htfs, 8)
        rp = resid(xu, imgs)
        t_plain.append(truth_err(xu, truth))
        x = ws.initial_volume(htfs)
        nd = np.full(len(rp), -1)
        cv, tv = [], []
        for k in range(0, 9):
            if k > 0:
                p.RichardsonLucy(hm, x, htfs, 1)
            rk = resid(x, imgs)
            cv.append(rk)
            tv.append(truth_err(x, truth))
            nd[(nd < 0) & (rk <= rp)] = k
        r_plain.append(rp)
        curves.append(np.stack(cv))
        tcurves.append(np.stack(tv))
        need.append(nd)
        del xu, x, truth
    r_plain = np.concatenate(r_plain)
    t_plain = np.concatenate(t_plain)
    curves = np.concatenate(curves, axis=1)
    tcurves = np.concatenate(tcurves, axis=1)
    curve = [float(v) for v in curves.mean(axis=1)]
    need = np.concatenate(need)
    k_warm = None if (need < 0).any() else int(need.max())
    img1 = imgs[:1].contiguous()
    htf1 = torch.empty((Z, 1, Y, X), device=dev)
    xp = torch.empty((Z, 1, Y, X), device=dev)

    def plain_step():
        ctx.backward(img1, htf1, 1, Y, X, None, stream=s.cuda_stream)
        xp.fill_(1.0)
        p.RichardsonLucy(hm, xp, htf1, 8)

    def warm_step():
        ctx.backward(img1, htf1, 1, Y, X, None, stream=s.cuda_stream)
        xw = ws.initial_volume(htf1)
        if k_warm:
            p.RichardsonLucy(hm, xw, htf1, k_warm)

    def timed(fn):
        for _ in range(max(args.warmup, 3)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(args.steps):
            fn()
        e1.record(s)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    # each arm's step replays one CUDA graph (back projection, network, RL iterations);
    # the direct launches are timed beside it
    saved = p.useGraphs
    p.useGraphs = False
    plain_step()
    torch.cuda.synchronize()
    g_plain = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g_plain, capture_error_mode="relaxed"):
        plain_step()
    p.useGraphs = saved
    g_warm = None
    if k_warm is not None:
        g_warm = warmstart.WarmStartGraph(ws, 1, k_warm)
        g_warm.img.copy_(img1)
    torch.cuda.synchronize()

    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)   # nvidia-smi's first sample
    clocks.mark(True)
    ms_plain = timed(g_plain.replay)
    ms_warm = timed(g_warm.replay) if g_warm is not None else None
    clocks.mark(False)
    clk = clocks.stop()
    ms_plain_direct = timed(plain_step)
    ms_warm_direct = timed(warm_step) if k_warm is not None else None
    net_ms = timed(lambda: ws.initial_volume(htf1))

    # kernel launches of one warm-start step: the projection kernels (launch
    # counters of the context) and the network's kernels, with the RL iterations
    # launched directly instead of from a graph
    p.useGraphs = False
    ctx.profile(False)
    n0 = _flf.net_launches()
    for _ in range(args.steps):
        warm_step()
    torch.cuda.synchronize()
    launches_warm = (sum(v["launches"] for v in ctx.profile_read().values()) + _flf.net_launches() - n0) / args.steps
    p.useGraphs = True

    # per-kernel times of the plain-RL arm: the same steps with every kernel
    # between CUDA events, on one stream (roofline of the multiply-accumulate)
    ctx.set_option("streams", 1)
    ctx.profile(True)
    for _ in range(args.steps):
        ctx.backward(img1, htf1, 1, Y, X, None, stream=s.cuda_stream)
        xp.fill_(1.0)
        ctx.rl_iterate(xp, htf1, None, _flf.FLF_RL_PREVEDEL, 8, 1, Y, X, stream=s.cuda_stream)
    torch.cuda.synchronize()
    prof = ctx.profile_read()
    ctx.profile(False)
    ctx.set_option("streams", 2)
    roof = mac_roofline(prof, survey_psf_bytes(N, Y, X, hs) * args.steps * 17,
                        "plain-RL arm, 17 projections per volume")

    # the network's dominant convolution (16 -> 16 channels at full resolution)
    # against the measured dense BF16 peak
    Zp, Yp, Xp = ws.pad
    g = torch.Generator(device=dev).manual_seed(0)
    xa = torch.randn((1, Zp, Yp, Xp, 16), generator=g, device=dev).bfloat16()
    wa = (torch.randn((27, 16, 16), generator=g, device=dev) / 20).bfloat16()
    ba = torch.zeros(16, device=dev)
    ya = torch.empty_like(xa)
    conv_ms = timed(lambda: _flf.conv3d(xa, wa, ba, ya, relu=True, stream=s.cuda_stream))
    _flf.net_status()
    flop = 2.0 * Zp * Yp * Xp * 27 * 16 * 16
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            bf16_peak, bf16_kind = float(json.load(f)["bf16_tflops"]), "measured (MEASURED_PEAKS.json bf16_tflops)"
    except Exception:
        bf16_peak, bf16_kind = 1900.0, "fallback"
    roof_net = {"bound": "tensor", "kernel": "k_conv3d_tma16 (16 -> 16 channels, tcgen05)", "unit": "TFLOP/s",
                "achieved": round(flop / conv_ms / 1e9, 1), "peak": bf16_peak, "peak_source": bf16_kind,
                "frac": round(flop / conv_ms / 1e9 / bf16_peak, 4), "avg_launch_ms": conv_ms,
                "flop_per_launch": flop, "shape": [Zp, Yp, Xp, 16]}
    del xa, ya

    # end to end through the public API: host image in, host volume out (pinned host buffers)
    img_h = pinned_like(img1)
    out = pinned_empty((Z, 1, Y, X))
    warmstart.DeconvRLWarm(ws, img_h, k_warm or 0, out=out, graph=True)
    torch.cuda.synchronize()
    ne = max(5, args.steps)
    t0 = time.perf_counter()
    for _ in range(ne):
        warmstart.DeconvRLWarm(ws, img_h, k_warm or 0, out=out, graph=True)
    e2e_s = (time.perf_counter() - t0) / ne
    fp64 = fp64_accuracy(wl["fp64_case"]) if wl.get("fp64_case") else None

    losses = [l for _, l in ws.losses]
    k_use = k_warm if k_warm is not None else 8
    line = {"metric": METRIC,
            "value": 1000.0 / ms_warm if ms_warm else 1000.0 / ms_plain, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms_warm or ms_plain,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 network (fp32 accumulation), f32 projections", "data": "synthetic",
            "config": {"workload": wl["label"], "image": [Y, X], "planes": Z, "nnum": N, "frames": 1,
                       "psf": psf_desc, "beads": wl["beads"], "filaments": wl.get("filaments", 0),
                       "train_steps": args.train_steps, "train_s": round(train_s, 1), "psf_s": round(psf_s, 1),
                       "conv_kernels": "tcgen05 for every layer, in training and inference",
                       "target_iters": args.target_iters, "residual_finetune_steps": args.tune_steps,
                       "residual_finetune_loss_first_last": ([ws.tune_losses[0][1], ws.tune_losses[-1][1]]
                                                             if ws.tune_losses else None),
                       "finetune_s": round(tune_s, 1),
                       "train_loss_mean_last_100": float(np.mean(losses[-100:])) if losses else None,
                       "train_loss_mean_first_100": float(np.mean(losses[:100])) if losses else None,
                       "network_parameters": ws.net.num_parameters(), "held_out_volumes": nseed,
                       "value_arm": "warm start" if ms_warm else "plain RL (the warm start missed the residual)",
                       "device_gb": round(ctx.memory_usage() / 1e9, 2),
                       "l2": "transfer matrices (%.2f GB per projection) and volumes larger than L2"
                             % (roof["own_bytes_per_launch"] * roof["launches"] / args.steps / 17 / 1e9)},
            "step_launch": "one CUDA graph per volume for each arm (ms_direct: the same kernels launched one by one)",
            "plain_rl": {"volumes_per_s": 1000.0 / ms_plain, "ms_per_volume": ms_plain, "iterations": 8,
                         "ms_direct": ms_plain_direct,
                         "residual_rel_l2_mean": float(r_plain.mean()),
                         "truth_rel_l2_scaled_mean": float(t_plain.mean())},
            "warm_start": {"rl_iterations_needed": k_warm, "network_ms": net_ms, "ms_direct": ms_warm_direct,
                           "residual_after_k_mean": [round(v, 5) for v in curve],
                           "truth_rel_l2_scaled_mean_after_k": [round(float(v), 5) for v in tcurves.mean(axis=1)],
                           "truth_rel_l2_scaled_mean": float(tcurves[k_use].mean()),
                           "speedup_vs_plain": (ms_plain / ms_warm) if ms_warm else None},
            "rl_iterations_per_s": 8 * 1000.0 / ms_plain,
            "accuracy": {"fp64": fp64, "residual_rel_l2_plain8_mean": float(r_plain.mean()),
                         "residual_rel_l2_warm_mean": float(curves[k_use].mean()), "reductions": "f64"},
            "e2e": {"value": 1.0 / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(img_h.nbytes),
                    "d2h_bytes_per_step": int(out.nbytes), "ms_per_step": e2e_s * 1000.0,
                    "path": "warmstart.DeconvRLWarm(graph=True) on a pinned host image, volume copied to pinned host memory"},
            "gpu_launches": int(round(launches_warm)), "roofline": roof, "roofline_network": roof_net,
            "cpu_baseline": cb, "clocks": clk}
    print(json.dumps(line), flush=True)


def run_config4(args):
    """Plain RL (8 Prevedel iterations from a uniform volume, after the back
    projection) of 16 frames per launch at Nnum 19 on 1919 x 1919 px images and
    51 planes, with the memory plan measured: the transfer matrices of both
    directions stay resident, the uploaded PSF quadrants are released after the
    precompute, and the volumes of the 16 frames are the only other large
    buffers.  One step = 16 deconvolved volumes."""
    import torch
    import _flf
    import build_lib
    import psfmatrix
    import projector
    import synthetic
    import warmstart
    build_lib.build()
    wl = WORKLOADS["config4"]
    N = wl["Nnum"]
    T = args.frames if args.frames > 1 else 16
    z0, z1, dz = wl["z"]
    z = np.arange(z0, z1 + dz / 2, dz)
    Z = len(z)
    Y = X = wl["lenslets"] * N
    dev = torch.device("cuda", 0)
    s = torch.cuda.current_stream(dev)
    t0 = time.time()
    hs = synthetic.psf_sizes(N, z, wl["img_size_ref"])
    nh = (N + 1) // 2

    class LazyPsf(psfmatrix.HMatrix):
        """The synthetic PSF set generated one plane at a time as the projector
        uploads it (the whole set is 36 GB of host memory)."""

        def __init__(self):
            super().__init__("mem:bench-config4/H{z:02d}", "mem:bench-config4/Ht{z:02d}",
                             [(nh, nh, h, h) for h in hs], cacheMMap=False)
            self._plane = (None, None)

        def Hcc(self, cc, useHt):
            if self._plane[0] != cc:
                H1, Ht1 = synthetic.synthetic_psf(N, z, wl["img_size_ref"], only=[cc])
                self._plane = (cc, (H1[cc], Ht1[cc]))
            return self._plane[1][1 if useHt else 0]

    hm = LazyPsf()
    psf_gb = 2 * sum(nh * nh * h * h * 4 for h in hs) / 1e9
    p = projector.Projector_gb300()
    p.storeVolumesOnGPU = True
    ctx = p.context(hm)
    hm._plane = (None, None)
    ctx.set_option("release_psf", 1)
    ctx.set_option("streams", args.streams)
    psf_s = time.time() - t0
    t1 = time.time()
    p._prepare(ctx, Y, X, hm)
    torch.cuda.synchronize()
    prep_s = time.time() - t1
    geo = ctx.geometry()
    mat_gb = ctx.memory_usage() / 1e9
    # synthetic frames rendered on the device and forward projected one at a time, Poisson noise
    rng = np.random.default_rng(4444)
    img = torch.empty((T, Y, X), device=dev)
    acc = torch.empty(Z * Y * X, dtype=torch.int64, device=dev)
    gt1 = None
    for t in range(T):
        g = torch.zeros((Z, 1, Y, X), device=dev)
        pts = torch.as_tensor(warmstart.synthetic_volume_points((Z, Y, X), wl["beads"], wl["filaments"], rng),
                              device=dev)
        _flf.render_blobs(g[:, 0], pts, 1.0, s.cuda_stream, acc=acc)
        ctx.forward(g, img[t:t + 1], 1, Y, X, None, stream=s.cuda_stream)
        if t == 0:
            gt1 = g[:, 0].cpu()
        del g
    del acc
    gen = torch.Generator(device=dev).manual_seed(55)
    img = torch.poisson((img + 100.0).clamp_min(0), generator=gen)
    htf = torch.empty((Z, T, Y, X), device=dev)
    x = torch.empty((Z, T, Y, X), device=dev)
    setup_s = time.time() - t0

    def step():
        ctx.backward(img, htf, T, Y, X, None, stream=s.cuda_stream)
        x.fill_(1.0)
        ctx.rl_iterate(x, htf, None, _flf.FLF_RL_PREVEDEL, args.iters, T, Y, X, stream=s.cuda_stream)

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    free_b, total_b = torch.cuda.mem_get_info(dev)
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    clocks.mark(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(args.steps):
        step()
    e1.record(s)
    torch.cuda.synchronize()
    clocks.mark(False)
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    ctx.synchronize(s.cuda_stream)
    # accuracy of frame 0: data-fit residual and error against its ground truth (FP64 reductions)
    hx = torch.empty((T, Y, X), device=dev)
    ctx.forward(x, hx, T, Y, X, None, stream=s.cuda_stream)
    torch.cuda.synchronize()
    y64, h64 = img[0].double(), hx[0].double()
    resid = float(torch.linalg.vector_norm(y64 - h64) / torch.linalg.vector_norm(y64))
    x0 = x[:, 0].double().cpu()
    g0 = gt1.double()
    a = float((x0 * g0).sum() / (x0 * x0).sum())
    truth = float(torch.linalg.vector_norm(a * x0 - g0) / torch.linalg.vector_norm(g0))
    line = {"metric": "volumes/s to plain-RL(8 it) accuracy, Nnum 19 full field, 16 frames per launch, 1 GB300",
            "value": T / (ms / 1000.0), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": max(1, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": wl["label"], "image": [Y, X], "planes": Z, "nnum": N, "frames": T,
                       "rl_iterations": args.iters, "psf_sizes_max": max(hs),
                       "psf": "synthetic set with the sizes of these optics (41 lenslets at 125 um)",
                       "transform_sizes": geo["f"], "precompute_fp64": geo["fp64"],
                       "psf_upload_s": round(psf_s, 1), "precompute_s": round(prep_s, 1),
                       "setup_s": round(setup_s, 1), "streams": args.streams,
                       "l2": "transfer matrices (%.0f GB per direction) streamed per projection" % (mat_gb / 2)},
            "memory": {"transfer_matrices_gb": round(mat_gb, 1), "psf_quadrants_gb_released": round(psf_gb, 1),
                       "library_gb_after_run": round(ctx.memory_usage() / 1e9, 1),
                       "device_used_gb": round((total_b - free_b) / 1e9, 1),
                       "torch_peak_allocated_gb": round(torch.cuda.max_memory_allocated(dev) / 1e9, 1),
                       "device_total_gb": round(total_b / 1e9, 1)},
            "rl_iterations_per_s": T * args.iters / (ms / 1000.0),
            "accuracy": {"frame": 0, "residual_rel_l2": resid, "truth_rel_l2_scaled": truth, "reductions": "f64"},
            "clocks": clk}
    print(json.dumps(line), flush=True)


def run_network_case(args):
    """The warm-start network's kernels on a random BF16 volume [1][Z][Y][X][C]
    (inputs larger than L2 at the default 24 x 456 x 456): one 16 -> 16 channel
    3x3x3 convolution with bias and ReLU (``conv16``), or the U-Net forward with
    its head (``unet``); CUDA-event time per call after the warm-up calls.  These
    are the cases the network kernel profiles are captured on."""
    import torch
    import build_lib
    import _flf
    build_lib.build()
    _flf.load_library()
    _flf.conv16_tcgen05({"mma.sync": 0, "tcgen05-all": 2}.get(args.kernel, 1))
    _flf.conv_wide_tcgen05(args.wide)
    Z, Y, X = args.shape
    g = torch.Generator(device="cuda").manual_seed(0)
    if args.workload == "conv16":
        x = torch.randn((1, Z, Y, X, 16), generator=g, device="cuda").bfloat16()
        w = (torch.randn((27, 16, 16), generator=g, device="cuda") / 20).bfloat16()
        b = torch.randn(16, generator=g, device="cuda")
        y = torch.empty_like(x)
        if args.kernel == "tcgen05-noswizzle":
            fn = lambda: _flf.conv3d_tc(x, w, b, y, relu=True, rows=0)   # noqa: E731
        else:
            fn = lambda: _flf.conv3d(x, w, b, y, relu=True)   # noqa: E731
        flop = 2.0 * Z * Y * X * 27 * 16 * 16
    else:
        import warmstart
        net = warmstart.UNet3D(seed=1)
        x = torch.zeros((1, Z, Y, X, warmstart.CIN), device="cuda").bfloat16()
        x[..., :4] = torch.rand((1, Z, Y, X, 4), generator=g, device="cuda").bfloat16()
        fn = lambda: net.forward(x)   # noqa: E731
        flop = None
    for _ in range(max(args.warmup, 3)):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    _flf.net_status()
    line = {"metric": "ms per call, %s" % WORKLOADS[args.workload]["label"], "value": ms, "unit": "ms",
            "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (fp32 accumulation)",
            "data": "synthetic", "config": {"workload": WORKLOADS[args.workload]["label"], "shape": [Z, Y, X],
                                            "kernel": args.kernel, "wide_kernel": args.wide,
                                            "l2": "activations larger than L2"}}
    if flop:
        line["tflops"] = flop / ms / 1e9
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "timeseries":
        run_timeseries(args)
    elif args.workload == "rectify":
        run_rectify(args)
    elif args.workload == "psf":
        run_psf(args)
    elif args.workload in ("warmstart", "warmstart_fullfield"):
        run_warmstart(args)
    elif args.workload in ("conv16", "unet"):
        run_network_case(args)
    elif args.workload == "config4":
        run_config4(args)
    else:
        run_gb300(args, rank, world, local)


if __name__ == "__main__":
    main()
