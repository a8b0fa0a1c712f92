#!/usr/bin/env python
"""Benchmark of the per-FOV image path (deconv + blur + maxima + fit).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mermake_gb300|reference]
                    [--workload fov3c|quad|ten|grid25|psfgrid|psfgrid9|tile|served|drift16]
                    [--form batched|plain] [--batch B]

A step is one FOV of the workload, inputs resident in HBM:

* ``fov3c`` (default): the full hyb FOV, 3 colours + DAPI, uint16
  50 x 2048 x 2048 per channel, 40,000 puncta per colour, quadratic flat
  field gain 0.8-1.0, DAPI of 300 nuclei; tile 500, overlap 89; hyb beta 1e-4,
  blur 30, threshold 3600, delta 1, fit 3, zpad 49; DAPI beta 0.01, blur 50,
  threshold 3.0, delta 5, fit 5, zpad 24.
* ``quad``: one colour of 50 x 1000 x 1000 (2 x 2 tiles), 10,000 puncta, flat
  field: the small case for profiler captures (spectra larger than L2).
* ``ten``: one colour of 50 x 1000 x 2500 (2 x 5 tiles of 500), flat field:
  the smallest batch that runs the z operator, for DRAM-traffic captures of
  every stage of the ``fov3c`` kernels (about 3 GB on the device).
* ``grid25``: one colour of 50 x 1000 x 1000 in 5 x 5 tiles of 200 (padded
  378): a 25-tile batch, like a colour of ``fov3c``, in a few GB.
* ``psfgrid``: one colour of 40 x 3000 x 3000 in tiles of 300 (padded 478),
  each of the 100 tiles with its own PSF from a 10 x 10 grid (sigma growing
  across the field), 60,000 puncta.
* ``psfgrid9``: the same per-tile PSFs on 40 x 900 x 900 (3 x 3 tiles, 3 x 3
  PSF grid): the small case for profiler captures of the PSF-grid kernels.
* ``tile``: one smFISH tile, uint16 40 x 500 x 500, 2,000 puncta, no flat field.
* ``served``: a Poisson stream (mean ``--interval``, 1.5 s) of ``--fovs``
  requests over 20 FOV ids whose shapes are drawn once per id (Z in
  {30, 40, 60, 80}, XY in {1024, 2048, 3000}, 1-4 colours + DAPI; FOV id =
  i mod 20, round = i div 20, later rounds drift-aligned against round 0)
  through ``serve.FovServer`` (continuous batching under a 120 GB budget);
  reports stream voxels/s and p50/p99 request latency.
* ``loader``: one 3-colour + DAPI FOV written in the acquisition's layout (bz2
  zarr of uint8 square-root frames, the xml's channel count) and read
  ``--steps`` times by ``io.FovPrefetcher`` (chunks decoded by a pool of host
  threads into pinned memory); reports FOV/s and decode GB/s on the host cores.
* ``drift16``: 16 DAPI rounds of one 50 x 2048 x 2048 field drifted by known
  shifts (+-3 z, +-20 x/y, sub-pixel), each deconvolved, spot-called and
  aligned against round 0's resident maxima; reports rounds/s and the error
  against the known shifts.

``value`` is FOV input voxels per second (all channels) of the batched form
(tiles of a colour in one batch, spots kept and offset on the device);
``--form plain`` times the per-tile loop of ``Deconvolver.tile_wise`` +
``find_local_maxima`` instead; ``--form graph`` replays the whole FOV captured
once as a CUDA graph (``pipeline.FovGraph``) on the resident channels.  ``e2e`` is the same metric through the same
public calls with the channels copied from pinned host memory every step and
the spot tables read back; in the batched form through ``pipeline.FovRunner``,
which copies the next FOV on a side stream while the current one computes.  ``roofline`` reports the dominant kernel (largest
share of device time in the timed region) from the library's per-stage CUDA
events, against the measured HBM copy bandwidth.  ``--impl reference`` times
the CPU restatement of the reference's functions (FP64 NumPy/SciPy FFT
deconvolution + C maxima/fit) on a bounded sample on the host cores.
"""
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

L2_BYTES = 129 * 2 ** 20

WORKLOADS = {
    "fov3c": dict(Z=50, X=2048, Y=2048, colours=3, puncta=40000, flat=True, dapi=True, nuclei=300,
                  hyb=dict(tile_size=500, overlap=89, beta=1e-4, threshold=3600, blur_radius=30, delta=1,
                           delta_fit=3, sigmaZ=1, sigmaXY=1.5),
                  dapi_args=dict(tile_size=500, overlap=89, beta=0.01, threshold=3.0, blur_radius=50, delta=5,
                                 delta_fit=5, sigmaZ=1, sigmaXY=1.5)),
    "fov80": dict(Z=80, X=2048, Y=2048, colours=3, puncta=40000, flat=True, dapi=True, nuclei=300,
                  hyb=dict(tile_size=500, overlap=89, beta=1e-4, threshold=3600, blur_radius=30, delta=1,
                           delta_fit=3, sigmaZ=1, sigmaXY=1.5),
                  dapi_args=dict(tile_size=500, overlap=89, beta=0.01, threshold=3.0, blur_radius=50, delta=5,
                                 delta_fit=5, sigmaZ=1, sigmaXY=1.5)),
    "dapi1k": dict(Z=50, X=1024, Y=1024, colours=0, puncta=0, flat=False, dapi=True, nuclei=75,
                   hyb=dict(tile_size=500, overlap=89, beta=1e-4, threshold=3600, blur_radius=30, delta=1,
                            delta_fit=3, sigmaZ=1, sigmaXY=1.5),
                   dapi_args=dict(tile_size=500, overlap=89, beta=0.01, threshold=3.0, blur_radius=50, delta=5,
                                  delta_fit=5, sigmaZ=1, sigmaXY=1.5)),
    "quad": dict(Z=50, X=1000, Y=1000, colours=1, puncta=10000, flat=True, dapi=False, nuclei=0,
                 hyb=dict(tile_size=500, overlap=89, beta=1e-4, threshold=3600, blur_radius=30, delta=1,
                          delta_fit=3, sigmaZ=1, sigmaXY=1.5)),
    "ten": dict(Z=50, X=1000, Y=2500, colours=1, puncta=25000, flat=True, dapi=False, nuclei=0,
                hyb=dict(tile_size=500, overlap=89, beta=1e-4, threshold=3600, blur_radius=30, delta=1,
                         delta_fit=3, sigmaZ=1, sigmaXY=1.5)),
    "grid25": dict(Z=50, X=1000, Y=1000, colours=1, puncta=10000, flat=True, dapi=False, nuclei=0,
                   hyb=dict(tile_size=200, overlap=89, beta=1e-4, threshold=3600, blur_radius=30, delta=1,
                            delta_fit=3, sigmaZ=1, sigmaXY=1.5)),
    "psfgrid": dict(Z=40, X=3000, Y=3000, colours=1, puncta=60000, flat=False, dapi=False, nuclei=0, psf_grid=10,
                    hyb=dict(tile_size=300, overlap=89, beta=1e-4, threshold=3600, blur_radius=30, delta=1,
                             delta_fit=3, sigmaZ=1, sigmaXY=1.5)),
    "psfgrid9": dict(Z=40, X=900, Y=900, colours=1, puncta=5400, flat=False, dapi=False, nuclei=0, psf_grid=3,
                     hyb=dict(tile_size=300, overlap=89, beta=1e-4, threshold=3600, blur_radius=30, delta=1,
                              delta_fit=3, sigmaZ=1, sigmaXY=1.5)),
    "tile": dict(Z=40, X=500, Y=500, colours=1, puncta=2000, flat=False, dapi=False, nuclei=0,
                 hyb=dict(tile_size=500, overlap=89, beta=1e-4, threshold=3600, blur_radius=30, delta=1,
                          delta_fit=3, sigmaZ=1, sigmaXY=1.5)),
}


for _name, _w in WORKLOADS.items():
    _w["name"] = _name

METRIC = "FOV voxels/s deconv+blur+maxima+fit"
DATA = "synthetic (seeded Poisson background + Gaussian puncta / nuclei, shapes of the named workload)"


def config_of(w, args, world):
    """The workload's config (the same dict on both arms)."""
    return {"workload": args.workload, "form": args.form, "Z": w["Z"], "X": w["X"], "Y": w["Y"],
            "channels": w["colours"] + (1 if w["dapi"] else 0), "tile_size": w["hyb"]["tile_size"],
            "overlap": w["hyb"]["overlap"], "fov_voxels": fov_voxels(w), "batch": args.batch,
            "l2": "inputs larger than L2 (%.2f GB per FOV vs 129 MB)" % (fov_voxels(w) * 2 / 1e9),
            "parallelism": "replicas" if world > 1 else "single", "zform": args.zform}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mermake_gb300", choices=["mermake_gb300", "reference"])
    ap.add_argument("--workload", default="fov3c", choices=sorted(WORKLOADS) + ["served", "drift16", "loader"])
    ap.add_argument("--fovs", type=int, default=200,
                    help="served: requests in the stream (FOV id = i mod 20, round = i div 20)")
    ap.add_argument("--interval", type=float, default=1.5, help="served: mean Poisson arrival interval (s)")
    ap.add_argument("--workers", type=int, default=2, help="served: concurrent requests on the device")
    ap.add_argument("--form", default="batched", choices=["batched", "plain", "graph"])
    ap.add_argument("--batch", type=int, default=0,
                    help="batched form: tiles per batch (0: the tuned / L2-rule size, -1: all tiles)")
    ap.add_argument("--zform", default="auto",
                    choices=["auto", "registers", "shared", "direct", "transforms", "tensor"],
                    help="z step form of every batch that qualifies for it (the library's MM_OPT_ZFORM)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="batched form: skip the plain-form, graph-form and parity blocks of the line")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


def fov_voxels(w):
    return (w["colours"] + (1 if w["dapi"] else 0)) * w["Z"] * w["X"] * w["Y"]


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def setup(w, device, seed=1000):
    import torch

    from mermake_gb300 import deconvolver, synth
    Z, X, Y = w["Z"], w["X"], w["Y"]
    psf = synth.gaussian_psf((40, 40, 40), 2.0, 1.3)
    if w.get("psf_grid"):
        # a PSF per tile in tile (x-major) order; sigma grows linearly across the field
        n = w["psf_grid"]
        psf = {(i, j): synth.gaussian_psf((40, 40, 40), 1.8 + 0.6 * (i + j) / (2 * n - 2),
                                          1.1 + 0.5 * (i + j) / (2 * n - 2)) for i in range(n) for j in range(n)}
    gain = synth.flat_gain(X, Y) if w["flat"] else None
    chans, flats = [], []
    for c in range(w["colours"]):
        chans.append(synth.hyb_stack(Z, X, Y, w["puncta"], seed + 17 * c, device=device, gain=gain))
        flats.append(torch.from_numpy(gain).to(device) if gain is not None else None)
    dapi = None
    if w["dapi"]:
        dapi = synth.dapi_stack(Z, X, Y, seed + 99, device=device, n_nuclei=w["nuclei"])
    dec_h = deconvolver.Deconvolver(psf, (Z, X, Y), zpad=Z - 1, **w["hyb"])
    dec_d = deconvolver.Deconvolver(psf, (Z, X, Y), zpad=(Z - 1) // 2, **w["dapi_args"]) if w["dapi"] else None
    torch.cuda.synchronize()
    return dict(chans=chans, flats=flats, dapi=dapi, dec_h=dec_h, dec_d=dec_d, w=w)


def run_fov(s, form, chans=None, dapi=None):
    """One FOV through the public API; returns the spot tables (device)."""
    import torch

    from mermake_gb300 import maxima, pipeline
    w = s["w"]
    chans = s["chans"] if chans is None else chans
    dapi = s["dapi"] if dapi is None else dapi
    if form == "graph":
        # one replay of the captured FOV (DAPI block and colours) on the
        # graph's resident inputs
        g = s["graph"]
        g.replay()
        got = g.results()
        if got is None:
            raise RuntimeError("a graph output overflowed")
        plus, minus, rows = got
        return ([plus, minus] if plus is not None else []) + rows
    out = []
    if w["dapi"]:
        p, m, buf, _ = pipeline.dapi_spots(s["dec_d"], dapi, None, buffer=s.get("buffer"), batch=s["batch"],
                                           **w["dapi_args"])
        s["buffer"] = buf
        out += [p, m]
    for c, ch in enumerate(chans):
        if form == "batched":
            out.append(pipeline.hyb_spots(s["dec_h"], ch, s["flats"][c], batch=s["batch"], **w["hyb"]))
        else:
            ov = w["hyb"]["overlap"]
            rows = []
            for x, y, tile, raw in s["dec_h"].tile_wise(ch, s["flats"][c], **w["hyb"]):
                Xh = maxima.find_local_maxima(tile, raw=raw, **w["hyb"])
                lim = torch.tensor([tile.shape[1] - ov, tile.shape[2] - ov], device=Xh.device)
                keep = torch.all((Xh[:, 1:3] >= ov) & (Xh[:, 1:3] < lim), dim=-1)
                if torch.any(keep):
                    Xh = Xh[keep]
                    Xh[:, 1] += x - ov
                    Xh[:, 2] += y - ov
                    rows.append(Xh)
            out.append(torch.cat(rows) if rows else torch.zeros((0, 8), device=ch.device))
    return out


def max_over_ranks(x, pg, device="cpu"):
    """The largest of the ranks' x (a replica job's time is its slowest rank's);
    pg: torch.distributed (any backend) or None for one process."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if pg is not None:
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, units_per_rank, steps, total_ms):
    """Whole-job units per second: each of the world replicas processed
    units_per_rank per step, the job took total_ms (its slowest rank)."""
    return world * units_per_rank * steps / (total_ms / 1e3)


def zpass_flops(w, s, zform="auto"):
    """FP32 flops of one FOV's z passes, by the form each channel's batch runs
    (the library's choice in run_tiles): one Z x Z complex matrix per frequency
    and tile when one spectrum serves a batch of >= 10 tiles of height <= 64,
    or when each tile's matrix is formed from its own z kernel (Z a multiple
    of 5 up to 80, 1 <= zpad <= Z - 1); else the direct sum over the padded
    planes (outputs and planes in blocks of 8).  A complex FMA is 8 flops."""
    shape = (w["Z"], w["X"], w["Y"])
    out = 0.0
    for dec, n in ((s["dec_h"], w["colours"]), (s["dec_d"], 1 if s["dec_d"] is not None else 0)):
        if not n:
            continue
        nt, Z, plane = dec.n_tiles(shape), dec.tile_height, dec.P * dec.H
        if dec.z_operator is None:
            continue
        shared = dec.psf_fft.shape[0] == 1 and nt >= 10 and Z <= 64
        per_tile = Z % 5 == 0 and Z <= 80 and 1 <= dec.zpad <= Z - 1
        if zform != "direct" and (shared or per_tile):
            per = Z * Z
        else:
            per = -(-Z // 8) * 8 * (-(-dec.Zp // 8) * 8)
        out += n * nt * plane * per * 8.0
    return out


def timed(fn, K, W, barrier, before_timed=None):
    import torch
    for _ in range(W):
        fn()
    if before_timed:
        before_timed()
    barrier()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(K + 1)]
    evs[0].record(st)
    for k in range(K):
        fn()
        evs[k + 1].record(st)
    torch.cuda.synchronize()
    barrier()
    per = [evs[k].elapsed_time(evs[k + 1]) for k in range(K)]
    return evs[0].elapsed_time(evs[K]), per


def pct(v, q):
    v = sorted(v)
    i = min(len(v) - 1, max(0, int(round(q / 100.0 * (len(v) - 1)))))
    return v[i]


def gpu_arm(args, rank, world, local):
    import torch

    from mermake_gb300 import _lib
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = WORKLOADS[args.workload]
    if args.zform != "auto":
        _lib.zform(["auto", "registers", "shared", "direct", "transforms", "tensor"].index(args.zform),
                   local).__enter__()
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
        pg = dist

    def barrier():
        if pg:
            pg.barrier()

    s = setup(w, dev, seed=1000 + rank)
    s["batch"] = args.batch
    if args.form == "graph":
        from mermake_gb300 import pipeline
        # sizes the rows from an eager FOV, then captures on the resident channels
        run_fov(s, "batched")
        torch.cuda.synchronize()
        s["graph"] = pipeline.FovGraph(s["dec_h"], s["dec_d"], (w["Z"], w["X"], w["Y"]), w["colours"], w["hyb"],
                                       w.get("dapi_args"), flats=s["flats"], batch=args.batch,
                                       inputs=(s["dapi"], s["chans"]))
    vox = fov_voxels(w)

    # device-resident timed region, with per-stage events live
    n0 = [0]

    def start_counting():
        # per-stage events and the launch count cover the timed steps only
        torch.cuda.synchronize()
        _lib.profile_enable(True)
        n0[0] = _lib.launch_count()

    with ClockSampler(local) as clk:
        total_ms, per = timed(lambda: run_fov(s, args.form), args.steps, args.warmup, barrier, start_counting)
    launches = _lib.launch_count() - n0[0]
    if args.form == "graph":  # replays bypass the host-side launch counter
        launches += s["graph"].launches * args.steps
    prof = _lib.profile_read()
    _lib.profile_enable(False)
    spots = [int(o.shape[0]) for o in run_fov(s, args.form)]
    total_ms = max_over_ranks(total_ms, pg, dev)
    ms_step = total_ms / args.steps
    value = job_rate(world, vox, args.steps, total_ms)

    # dominant kernel (the graph form records no per-stage events: its line
    # points at the batched form's roofline, the same kernels)
    stages = {k: v for k, v in prof.items() if v[2] > 0}
    dom = max(stages, key=lambda k: stages[k][0]) if stages else None
    dms, dbytes, dl = stages[dom] if stages else (0.0, 0.0, 1)
    peaks = {}
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        peaks = json.load(open(pp))
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    achieved = (dbytes / dl) / ((dms / dl) / 1e3) / 1e9 if stages else None
    # DRAM traffic of the dominant kernel per launch: ncu's bytes per tile on
    # the ten-tile workload, scaled by the tiles one launch of this run processes
    traffic = None
    tp = os.path.join(ROOT, "profiles", "dram_traffic_ten.json")
    if os.path.exists(tp):
        e = json.load(open(tp))["stages"].get(dom) if dom else None
        if e:
            shape = (w["Z"], w["X"], w["Y"])
            tiles = len(s["dec_h"].tile_boxes(shape)) * w["colours"]
            if s["dec_d"] is not None:
                tiles += len(s["dec_d"].tile_boxes(shape))
            traffic = e["per_tile"] * tiles * args.steps / dl + e["per_launch"]
    stage_share = {k: round(v[0] / sum(x[0] for x in stages.values()), 4) for k, v in stages.items()} if stages else {}

    line = {
        "metric": METRIC,
        "value": value,
        "unit": "voxels/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": DATA,
        "config": config_of(w, args, world),
        "latency_ms": {"p50": pct(per, 50), "p99": pct(per, 99)},
        "spots_per_fov": spots,
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved else None, "peak_source": peak_src, "traffic": traffic,
                     "traffic_source": "profiles/dram_traffic_ten.json scaled by tiles per launch" if traffic else None,
                     "bytes_per_launch": dbytes / dl if stages else None, "ms_per_launch": dms / dl if stages else None,
                     "stage_share": stage_share} if stages else
                    {"note": "no per-stage events inside the graph; the batched form's line has the roofline"},
        "clocks": clk.summary(),
    }
    if dom == "zpass" and args.form == "batched":
        # the z pass is bound by FP32 FMA issue, not by bytes: the line's bound
        # is its arithmetic against the nominal FP32 peak (SMs x 128 lanes x 2
        # flops x the sampled maximum SM clock; the measured peaks file has no
        # FP32 figure), with the HBM figures beside it
        props = torch.cuda.get_device_properties(dev)
        mhz = (line["clocks"] or {}).get("sm_max_mhz") or peaks.get("sm_max_mhz") or 2070.0
        fpeak = props.multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12
        fl = zpass_flops(w, s, args.zform) * args.steps / dl
        fach = fl / ((dms / dl) / 1e3) / 1e12
        rf = line["roofline"]
        hbm = {k: rf[k] for k in ("achieved", "peak", "unit", "frac", "peak_source")}
        rf.update(bound="fp32", achieved=fach, peak=fpeak, unit="TFLOP/s", frac=fach / fpeak,
                  peak_source="nominal (SMs x 128 FP32 lanes x 2 x max SM clock)", flops_per_launch=fl, hbm=hbm)

    if not args.no_e2e:
        import torch

        from mermake_gb300 import pipeline
        host_ch = [c.cpu().pin_memory() for c in s["chans"]]
        host_dapi = s["dapi"].cpu().pin_memory() if s["dapi"] is not None else None
        io = {"h2d": 0, "d2h": 0}
        if args.form == "batched":
            # the public FovRunner: FOV k+1's channels are copied from pinned host
            # memory on a side stream while FOV k computes, and FOV k is launched
            # before FOV k - 1's rows are collected, so the GPU has work queued
            # while the host reads results.  Every step copies one FOV, launches
            # one and reads one back; the timed region ends after the last FOV
            # it launched and the last copy it issued.
            runner = pipeline.FovRunner(s["dec_h"], s["dec_d"], w["hyb"], w.get("dapi_args"), batch=args.batch)
            state = {}

            def e2e_step():
                t = state.pop("next", None) or runner.submit(host_dapi, host_ch)
                pend = runner.launch(t, s["flats"])
                prev = state.pop("pending", None)
                if prev is not None:
                    p, m, rows = runner.collect(prev)
                    io["d2h"] = sum(a.nbytes for a in [p, m] + rows if a is not None)
                state["pending"] = pend
                state["next"] = runner.submit(host_dapi, host_ch)
                io["h2d"] = runner.h2d_bytes

            for _ in range(max(args.warmup, 1)):
                e2e_step()
            torch.cuda.synchronize()
            barrier()
            st = torch.cuda.current_stream()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(args.steps):
                e2e_step()
            st.wait_stream(runner.copy_stream)
            e1.record(st)
            torch.cuda.synchronize()
            barrier()
            e_ms = e0.elapsed_time(e1)
            runner.collect(state.pop("pending"))
        else:
            if args.form == "graph":  # the graph reads the channels it was captured on
                dev_ch, dev_dapi = s["chans"], s["dapi"]
            else:
                dev_ch = [torch.empty_like(c) for c in s["chans"]]
                dev_dapi = torch.empty_like(s["dapi"]) if s["dapi"] is not None else None

            def e2e_step():
                for h, d in zip(host_ch, dev_ch):
                    d.copy_(h, non_blocking=True)
                if host_dapi is not None:
                    dev_dapi.copy_(host_dapi, non_blocking=True)
                outs = run_fov(s, args.form, chans=dev_ch, dapi=dev_dapi)
                hb = [o.to("cpu") for o in outs]
                io["h2d"] = sum(h.numel() * h.element_size() for h in host_ch) + (
                    host_dapi.numel() * host_dapi.element_size() if host_dapi is not None else 0)
                io["d2h"] = sum(h.numel() * h.element_size() for h in hb)

            e_ms, _ = timed(e2e_step, args.steps, 1, barrier)
        e_ms = max_over_ranks(e_ms, pg, dev)
        line["e2e"] = {"value": job_rate(world, vox, args.steps, e_ms), "unit": "voxels/s",
                       "h2d_bytes_per_step": io["h2d"], "d2h_bytes_per_step": io["d2h"],
                       "ms_per_step": e_ms / args.steps}

    if args.form == "batched" and world == 1 and not args.no_extra:
        line["vs_plain"] = plain_block(s, ms_step, barrier)
        line["graph"] = graph_block(s, w, args, ms_step, spots, barrier)
        line["parity"] = parity_block(w, s)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, s)
    if pg:
        pg.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def plain_block(s, batched_ms, barrier, fovs=2):
    """The plain per-tile form of the same FOV (Deconvolver.tile_wise, then
    find_local_maxima and the keep/offset step per tile, the loop of
    mermake/__main__.py:253-265, on this library's kernels), timed like the
    batched form on the resident channels."""
    total, per = timed(lambda: run_fov(s, "plain"), fovs, 1, barrier)
    ms = total / fovs
    return {"form": "plain per-tile loop (tile_wise + find_local_maxima + keep/offset per tile)",
            "fovs": fovs, "ms_per_fov": ms, "ratio": ms / batched_ms}


def graph_block(s, w, args, batched_ms, spots, barrier):
    """The whole FOV captured once as a CUDA graph (pipeline.FovGraph) on the
    resident channels, replayed per FOV; the spot counts must equal the
    batched form's."""
    import torch

    from mermake_gb300 import pipeline
    with pipeline.FovGraph(s["dec_h"], s["dec_d"], (w["Z"], w["X"], w["Y"]), w["colours"], w["hyb"],
                           w.get("dapi_args"), flats=s["flats"], batch=args.batch,
                           inputs=(s["dapi"], s["chans"])) as g:
        gs = dict(s, graph=g)
        total, per = timed(lambda: run_fov(gs, "graph"), args.steps, args.warmup, barrier)
        counts = [int(o.shape[0]) for o in run_fov(gs, "graph")]
        torch.cuda.synchronize()
        ms = total / args.steps
        return {"ms_per_fov": ms, "ratio_vs_batched": batched_ms / ms, "library_launches_per_fov": g.launches,
                "fallbacks": g.fallbacks, "spots_equal_batched": counts == spots,
                "latency_ms": {"p50": pct(per, 50), "p99": pct(per, 99)}}


# ---------------------------------------------------------------------------
# CPU restatement of the reference (oracle) on a bounded sample
# ---------------------------------------------------------------------------
_ORACLE_W = {}


def oracle_W(key, make):
    if key not in _ORACLE_W:
        _ORACLE_W[key] = make()
    return _ORACLE_W[key]


def interior_tile(w, a):
    """Index (x-major) of the tile at the second origin in x and y (the first
    interior tile when the axis has more than one), else 0."""
    ts = a["tile_size"]
    ny = -(-w["Y"] // ts)
    return (1 if w["X"] > ts else 0) * ny + (1 if w["Y"] > ts else 0)


def owned_voxels(w, a, box):
    """The channel voxels a tile accounts for: its tile_size square, clipped."""
    ts = a["tile_size"]
    return w["Z"] * min(ts, w["X"] - box[0]) * min(ts, w["Y"] - box[1])


def oracle_hyb_tile(w, img_np, flat_np, psf, t):
    """The oracle on hyb tile t (Deconvolver.tile_wise + find_local_maxima,
    mermake/deconvolver.py:98-170, mermake/maxima.py:17-98): FP64 scipy.fft
    deconvolution and blur, C maxima + fit.  Returns (box, res, raw, Xh) with
    Xh in tile coordinates (before the keep filter)."""
    import numpy as np

    from oracle import ckernels as ck
    from oracle import deconv as od
    a, Z = w["hyb"], w["Z"]
    W = oracle_W(("hyb", Z, a["tile_size"], a["overlap"], a["beta"]),
                 lambda: od.wiener_half(psf, Z, a["tile_size"], Z - 1, a["overlap"], a["beta"]))
    box = od.tiles(img_np.shape, a["tile_size"], a["overlap"])[t]
    res, raw = od.deconv_tile(img_np, flat_np, box, W, a["tile_size"], Z - 1, a["overlap"], a["blur_radius"])
    Xh = ck.find_local_maxima(res.astype(np.float32), a["threshold"], a["delta"], a["delta_fit"], raw, a["sigmaZ"],
                              a["sigmaXY"])
    return box, res, raw, Xh


def oracle_dapi_tile(w, dapi_np, psf, t):
    """The oracle's DAPI block (mermake/__main__.py:215-225) on the region tile t
    stitches: FP64 deconvolution and blur of the tile, its centre as
    Deconvolver.apply writes it, divided by the RMS (here the region's own),
    maxima + fit of v and -v with the uint16 channel as raw.  Returns the
    region's voxels and the two row sets."""
    import numpy as np

    from oracle import ckernels as ck
    from oracle import deconv as od
    a, Z = w["dapi_args"], w["Z"]
    zpad, ov = (Z - 1) // 2, a["overlap"]
    W = oracle_W(("dapi", Z, a["tile_size"], ov, a["beta"]),
                 lambda: od.wiener_half(psf, Z, a["tile_size"], zpad, ov, a["beta"]))
    box = od.tiles(dapi_np.shape, a["tile_size"], ov)[t]
    res, _ = od.deconv_tile(dapi_np, None, box, W, a["tile_size"], zpad, ov, a["blur_radius"])
    xe, ye = res.shape[1:]
    cen = np.ascontiguousarray(res[:, ov:xe - ov, ov:ye - ov], dtype=np.float32)
    rms = np.float32(np.float32(np.sqrt((cen.astype(np.float64) ** 2).sum())) / np.sqrt(cen.size))
    v = cen / rms
    x, y = box[:2]
    raw = np.ascontiguousarray(dapi_np[:, x:x + cen.shape[1], y:y + cen.shape[2]], dtype=np.float32)
    Xp = ck.find_local_maxima(v, a["threshold"], a["delta"], a["delta_fit"], raw, a["sigmaZ"], a["sigmaXY"])
    Xm = ck.find_local_maxima(-v, a["threshold"], a["delta"], a["delta_fit"], raw, a["sigmaZ"], a["sigmaXY"])
    return cen.size, Xp, Xm


def keep_offset(Xh, box, extent, ov):
    """mermake/__main__.py:253-260 on one tile's rows (float32 arithmetic)."""
    import numpy as np
    xe, ye = extent
    Xh = np.array(Xh, dtype=np.float32, copy=True)
    k = np.all((Xh[:, 1:3] >= ov) & (Xh[:, 1:3] < np.array([xe - ov, ye - ov], np.float32)), axis=-1)
    Xh = Xh[k]
    Xh[:, 1] += np.float32(box[0] - ov)
    Xh[:, 2] += np.float32(box[1] - ov)
    return Xh


KEEP_MARGIN = 2e-3  # px: keep decisions closer than this to a boundary fall to rounding


def tile_window(R, box, extent, ov, margin=0.0):
    """Rows of a colour whose FOV centroids fall in the region a tile keeps,
    shrunk by ``margin`` on every side."""
    x, y = box[:2]
    xe, ye = extent
    return R[(R[:, 1] >= x + margin) & (R[:, 1] < x + xe - 2 * ov - margin) & (R[:, 2] >= y + margin)
             & (R[:, 2] < y + ye - 2 * ov - margin)]


def parity_block(w, s):
    """Parity of the timed configuration on one interior tile of colour 0.
    The tile's volume is taken from the production batch (the same batch size,
    so the same z form), with the truncated box blur of tile_wise (compared
    with the FP64 oracle over the whole yielded view) and with the blur folded
    into the z step as the drivers run it (compared over the voxels at least
    the box half-width from the tile edges, all the drivers read); the
    oracle's C maxima + fit on the drivers' volume (keep filter, offset) are
    compared with the batched driver's rows in the tile's region: the same
    maxima, centroids within 1e-3 px, heights within 1e-4 relative.  The
    oracle's rows on its own FP64 volume are reported beside them (maxima
    close to the threshold can flip with float32 rounding)."""
    import numpy as np
    import torch

    from mermake_gb300 import _lib, deconvolver, pipeline, synth, tune
    from oracle import ckernels as ck
    a, dec = w["hyb"], s["dec_h"]
    ch, fl = s["chans"][0], s["flats"][0]
    shape = tuple(int(v) for v in ch.shape)
    nt = dec.n_tiles(shape)
    t = interior_tile(w, a)
    b = tune.batch_for(dec, shape) if s["batch"] == 0 else s["batch"]
    nb = nt if b <= 0 else b
    t0 = (t // nb) * nb
    n = min(nb, nt - t0)
    box = dec.tile_boxes(shape)[t]
    ext = dec._extent(box)
    res = torch.empty((n, w["Z"], dec.P, dec.P), dtype=torch.float32, device=ch.device)
    raw = torch.empty_like(res)
    vols = {}
    # the truncated box blur of tile_wise, and the drivers' form (the blur
    # subtraction folded into the z step): the volumes the timed FOVs computed
    for mode in (_lib.MM_BLUR_EXACT, _lib.MM_BLUR_SPECTRAL):
        with _lib.blur_mode(mode):
            dec._call(ch, deconvolver.MM_DTYPE_U16, fl, t0, n, a["blur_radius"], res_out=res, raw_out=raw)
        vols[mode] = (res[t - t0, :, :ext[0], :ext[1]].cpu().numpy(), raw[t - t0, :, :ext[0], :ext[1]].cpu().numpy())
    del res, raw
    torch.cuda.empty_cache()
    g_res, g_raw = vols[_lib.MM_BLUR_SPECTRAL]
    rows = pipeline.hyb_spots(dec, ch, fl, batch=s["batch"], **a).cpu().numpy()
    img_np = ch.cpu().numpy()
    flat_np = fl.cpu().numpy() if fl is not None else None
    psf = synth.gaussian_psf((40, 40, 40), 2.0, 1.3)
    obox, o_res, o_raw, o_Xh = oracle_hyb_tile(w, img_np, flat_np, psf, t)
    assert tuple(obox) == tuple(box)
    scale = np.abs(o_res).max()
    err = float(np.abs(vols[_lib.MM_BLUR_EXACT][0].astype(np.float64) - o_res).max() / scale)
    d = a["blur_radius"] // 2
    inner = (slice(None), slice(d, min(ext[0], dec.P - d)), slice(d, min(ext[1], dec.P - d)))
    err_f = float(np.abs(g_res[inner].astype(np.float64) - o_res[inner]).max() / scale)
    ov = a["overlap"]
    want_all = keep_offset(ck.find_local_maxima(g_res, a["threshold"], a["delta"], a["delta_fit"], g_raw,
                                                a["sigmaZ"], a["sigmaXY"]), box, ext, ov)
    # rows whose centroid lies within KEEP_MARGIN of a keep boundary may be
    # kept by either side (a float centroid known to 1e-3 px); all others must agree
    got = tile_window(rows, box, ext, ov, KEEP_MARGIN)
    want = tile_window(want_all, box, ext, ov, KEEP_MARGIN)
    out = {"tile": t, "box": list(box), "extent": list(ext), "max_rel_voxel": err,
           "max_rel_voxel_folded_blur": err_f,
           "folded_blur_region": "voxels >= %d (the box half-width) from the padded tile's edges" % d,
           "voxel_tolerance": 1e-4, "raw_equal": bool(np.array_equal(g_raw, o_raw)), "rows_gpu": int(len(tile_window(rows, box, ext, ov))),
           "rows_oracle_on_gpu_volume": int(len(want_all)), "rows_compared": int(len(want)),
           "keep_margin_px": KEEP_MARGIN}
    try:
        g, wnt = ck.match_rows(got, want)
        dc = float(np.abs(g[:, :3] - wnt[:, :3]).max(initial=0.0))
        dh = float((np.abs(g[:, 7] - wnt[:, 7]) / np.maximum(np.abs(wnt[:, 7]), 1e-30)).max(initial=0.0))
        out.update(maxima_equal=True, max_centroid_diff_px=dc, max_rel_h=dh,
                   fit_within_tolerance=bool(dc <= 1e-3 + 2e-6 * float(np.abs(wnt[:, :3]).max(initial=0))
                                             and dh <= 1e-4))
    except AssertionError as e:
        out.update(maxima_equal=False, mismatch=str(e)[:200])
    o_rows = keep_offset(o_Xh, box, ext, ov)
    gi = {tuple(np.round(r[:3], 1)) for r in got}
    oi = {tuple(np.round(r[:3], 1)) for r in o_rows}
    out["rows_oracle_fp64"] = int(len(o_rows))
    out["fp64_rows_shared"] = len(gi & oi) / max(1, len(gi | oi))
    return out


def cpu_baseline(w, s=None, steps=1):
    """Times the oracle on an interior tile of each channel kind: one hyb tile
    (deconvolution + blur + maxima + fit) and, where the workload has a DAPI
    channel, the DAPI block on one tile's region (deconvolution, RMS, maxima
    and fit of both signs at delta 5).  The FOV time is extrapolated from the
    voxels each tile accounts for: colours x hyb + DAPI."""
    import numpy as np

    from mermake_gb300 import synth
    from oracle import build as obuild
    obuild.build_oracle()
    Z, X, Y = w["Z"], w["X"], w["Y"]
    a = w["hyb"]
    psf = synth.gaussian_psf((40, 40, 40), 2.0, 1.3)
    if s is not None:
        img = s["chans"][0].cpu().numpy()
        flat = s["flats"][0].cpu().numpy() if s["flats"][0] is not None else None
        dapi = s["dapi"].cpu().numpy() if s["dapi"] is not None else None
    else:
        gain = synth.flat_gain(X, Y) if w["flat"] else None
        img = synth.hyb_stack(Z, X, Y, w["puncta"], 1000, gain=gain).numpy()
        flat = gain
        dapi = synth.dapi_stack(Z, X, Y, 1099, n_nuclei=w["nuclei"]).numpy() if w["dapi"] else None
    t = interior_tile(w, a)
    oracle_hyb_tile(w, img, flat, psf, t)  # warm (Wiener spectrum, FFT plans)
    if dapi is not None:
        oracle_dapi_tile(w, dapi, psf, interior_tile(w, w["dapi_args"]))
    th = td = 0.0
    vh = vd = 0
    for _ in range(steps):
        t0 = time.perf_counter()
        box, _, _, _ = oracle_hyb_tile(w, img, flat, psf, t)
        th += time.perf_counter() - t0
        vh += owned_voxels(w, a, box)
        if dapi is not None:
            t0 = time.perf_counter()
            v, _, _ = oracle_dapi_tile(w, dapi, psf, interior_tile(w, w["dapi_args"]))
            td += time.perf_counter() - t0
            vd += v
    chan = Z * X * Y
    fov_s = w["colours"] * chan * th / vh + (chan * td / vd if dapi is not None else 0.0)
    P = a["tile_size"] + 2 * a["overlap"]
    sample = ("%d x (interior hyb tile %dx%d of the %s workload, padded %dx%dx%d: FP64 scipy.fft deconvolution + "
              "blur, C maxima/fit (OpenMP)" % (steps, a["tile_size"], a["tile_size"], w.get("name", ""), 3 * Z - 2, P, P))
    if dapi is not None:
        sample += ("; interior DAPI tile, padded %dx%dx%d: deconvolution + blur, RMS, maxima/fit of both signs at "
                   "delta 5" % (Z + 2 * ((Z - 1) // 2), P, P))
    sample += "); FOV time extrapolated per owned voxel: %d colours x hyb%s; Wiener spectra built untimed" % (
        w["colours"], " + DAPI" if dapi is not None else "")
    return {"value": fov_voxels(w) / fov_s, "unit": "voxels/s", "cores": os.cpu_count(), "kind": "port",
            "sample": sample, "seconds": th + td, "fov_seconds_extrapolated": fov_s,
            "hyb_tile_s": th / steps, "dapi_tile_s": td / steps if dapi is not None else None}


def reference_arm(args, rank, world):
    if rank != 0:
        return
    w = WORKLOADS[args.workload]
    cb = cpu_baseline(w, None, steps=max(1, args.steps))
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": cb["value"],
        "unit": "voxels/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": cb["fov_seconds_extrapolated"] * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": DATA,
        "config": config_of(w, args, world),
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# served form: a Poisson stream of mixed-shape FOVs through serve.FovServer
# ---------------------------------------------------------------------------
def served_fovs(n=20, seed=4):
    """(Z, X, Y, colours) of the stream's FOV ids, drawn once per id: Z in
    {30, 40, 60, 80}, XY in {1024, 2048, 3000}, 1-4 colours (plus DAPI)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        xy = int(rng.choice((1024, 2048, 3000)))
        out.append((int(rng.choice((30, 40, 60, 80))), xy, xy, int(rng.integers(1, 5))))
    return out


def served_arm(args, local):
    import numpy as np
    import torch

    from mermake_gb300 import serve, synth
    torch.cuda.set_device(local)
    hyb = dict(WORKLOADS["fov3c"]["hyb"])
    dap = dict(WORKLOADS["fov3c"]["dapi_args"])
    psf = synth.gaussian_psf((40, 40, 40), 2.0, 1.3)
    fovs = served_fovs()
    data = []
    for f, (Z, X, Y, nc) in enumerate(fovs):
        dapi = synth.dapi_stack(Z, X, Y, 500 + f, device="cuda", n_nuclei=max(20, 300 * X * Y // 2048 ** 2))
        gain = synth.flat_gain(X, Y)
        cols = [synth.hyb_stack(Z, X, Y, 40000 * X * Y // 2048 ** 2, 600 + 7 * f + c, device="cuda", gain=gain)
                for c in range(nc)]
        data.append(dict(dapi=dapi.cpu().pin_memory(), colours=[c.cpu().pin_memory() for c in cols],
                         flats=[torch.from_numpy(gain).cuda() for _ in cols]))
        del dapi, cols
    rng = np.random.default_rng(7)
    nf = len(fovs)
    reqs = [dict(fov=i % nf, round=i // nf, **data[i % nf]) for i in range(args.fovs)]
    vox = [sum(int(np.prod(a.shape)) for a in [r["dapi"]] + r["colours"]) for r in reqs]
    gaps = rng.exponential(args.interval, size=len(reqs))
    with ClockSampler(local) as clk:
        with serve.FovServer(psf, hyb, dap, hbm_budget=120e9, workers=args.workers) as srv:
            # warm-up: one request per shape builds the resident spectra (untimed)
            for f in range(nf):
                srv.submit(serve.FovRequest(fov=1000 + f, round=0, **data[f])).result()
            srv.results.clear()
            futs, t0 = [], time.perf_counter()
            t = t0
            for r, g in zip(reqs, gaps):
                t += g
                while time.perf_counter() < t:
                    time.sleep(min(0.002, max(0.0, t - time.perf_counter())))
                futs.append(srv.submit(serve.FovRequest(arrival=t, **r)))
            res = [fu.result() for fu in futs]
            t1 = max(x.done for x in res)
            peak = srv.max_in_flight
            peak_bytes, releases = srv.peak_bytes, srv.releases
    lat = sorted(1e3 * x.latency for x in res)
    svc = sorted(1e3 * (x.done - x.admitted) for x in res)
    que = sorted(1e3 * (x.admitted - x.request.arrival) for x in res)
    line = {
        "metric": "FOV voxels/s, served stream (Poisson arrivals, mixed Z/XY, continuous batching)",
        "value": sum(vox) / (t1 - t0),
        "unit": "voxels/s",
        "n_gpus": 1,
        "steps": len(reqs),
        "warmup": nf,
        "ms_per_step": 1e3 * (t1 - t0) / len(reqs),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded Poisson background + Gaussian puncta / nuclei), %d FOV shapes" % nf,
        "config": {"workload": "served", "fovs": [list(f) for f in fovs], "requests": len(reqs),
                   "mean_interval_s": args.interval, "workers": args.workers, "hbm_budget_gb": 120,
                   "peak_in_flight": peak, "peak_device_gb_held": peak_bytes / 1e9,
                   "idle_worker_releases": releases, "tile_size": hyb["tile_size"], "overlap": hyb["overlap"]},
        "latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99), "max": lat[-1]},
        "service_ms": {"p50": pct(svc, 50), "p99": pct(svc, 99)},
        "queue_ms": {"p50": pct(que, 50), "p99": pct(que, 99)},
        "per_fov_service_ms": {"%d: %s" % (f, list(fovs[f])): round(statistics.median(
            1e3 * (x.done - x.admitted) for x in res if x.request.fov == f), 1)
            for f in range(nf) if any(x.request.fov == f for x in res)},
        "drift_px": [float(np.abs(np.asarray(x.drift[0])).max()) for x in res if x.drift is not None][:8],
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# drift: 16 DAPI rounds of one FOV with known drifts against round 0
# ---------------------------------------------------------------------------
def drift_arm(args, local):
    import types

    import numpy as np
    import torch

    from mermake_gb300 import align, deconvolver, pipeline, synth
    torch.cuda.set_device(local)
    Z, X, Y = 50, 2048, 2048
    dap = dict(WORKLOADS["fov3c"]["dapi_args"])
    psf = synth.gaussian_psf((40, 40, 40), 2.0, 1.3)
    dec = deconvolver.Deconvolver(psf, (Z, X, Y), zpad=(Z - 1) // 2, **dap)
    rng = np.random.default_rng(11)
    shifts = [(0.0, 0.0, 0.0)] + [(rng.uniform(-3, 3), rng.uniform(-20, 20), rng.uniform(-20, 20))
                                  for _ in range(15)]
    rounds = [synth.dapi_stack(Z, X, Y, 900, device="cuda", offset=s, noise_seed=900 + r).cpu().pin_memory()
              for r, s in enumerate(shifts)]
    buf = [None]

    def maxima(h):
        p, m, buf[0], _ = pipeline.dapi_spots(dec, h.to("cuda", non_blocking=True), None, buffer=buf[0], **dap)
        return types.SimpleNamespace(Xh_plus=p, Xh_minus=m)

    ref = maxima(rounds[0])
    dual = align.DualAligner(ref, th=4)  # round 0's maxima stay on the device
    for r in range(1, 4):  # warm-up
        dual.get_best_translation_pointsV2(maxima(rounds[r]))
    torch.cuda.synchronize()
    errs, times = [], []
    with ClockSampler(local) as clk:
        for r in range(1, len(rounds)):
            t0 = time.perf_counter()
            tz = dual.get_best_translation_pointsV2(maxima(rounds[r]))[0]
            times.append(1e3 * (time.perf_counter() - t0))
            errs.append(np.asarray(tz, np.float64) + np.asarray(shifts[r]))
    errs = np.abs(np.array(errs))
    line = {
        "metric": "drift rounds/s (DAPI deconvolution + maxima + drift against round 0)",
        "value": 1e3 * len(times) / sum(times),
        "unit": "rounds/s",
        "n_gpus": 1, "steps": len(times), "warmup": 3,
        "ms_per_step": sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic DAPI field of 300 nuclei, drifted by known shifts (+-3 z, +-20 x/y, sub-pixel)",
        "config": {"workload": "drift16", "Z": Z, "X": X, "Y": Y, "rounds": len(rounds), "reference": "round 0"},
        "drift_error_px": {"max_z": float(errs[:, 0].max()), "max_x": float(errs[:, 1].max()),
                           "max_y": float(errs[:, 2].max()), "mean": float(errs.mean())},
        "latency_ms": {"p50": pct(sorted(times), 50), "p99": pct(sorted(times), 99)},
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# loader: the FOV reader with prefetch on the host cores
# ---------------------------------------------------------------------------
def write_fov_zarr(root, chans, fov="Conv_zscan__000", workers=None):
    """One FOV in the layout mermake/io.py:read_im reads: frames of uint8
    (the square root of the uint16 intensities, as the acquisition stores
    them), frame 0 a dummy, then the channels interleaved plane by plane,
    one bz2 (level 9) chunk per frame, and the xml's z_offsets naming the
    channel count."""
    import bz2
    import concurrent.futures as cf

    import numpy as np
    nch, (Z, X, Y) = len(chans), chans[0].shape
    d = os.path.join(root, fov.split("_")[-1], "data")
    os.makedirs(d, exist_ok=True)
    n = 1 + nch * Z
    json.dump({"chunks": [1, X, Y], "compressor": {"id": "bz2", "level": 9}, "dtype": "|u1", "fill_value": 0,
               "filters": None, "order": "C", "shape": [n, X, Y], "zarr_format": 2},
              open(os.path.join(d, ".zarray"), "w"))

    def frame(i):
        if i == 0:
            u8 = np.zeros((X, Y), np.uint8)
        else:
            c, z = (i - 1) % nch, (i - 1) // nch
            u8 = np.minimum(np.rint(np.sqrt(chans[c][z].astype(np.float32))), 255).astype(np.uint8)
        with open(os.path.join(d, "%d.0.0" % i), "wb") as f:
            f.write(bz2.compress(u8.tobytes(), 9))

    with cf.ThreadPoolExecutor(max_workers=workers or os.cpu_count()) as ex:
        list(ex.map(frame, range(n)))
    with open(os.path.join(root, fov + ".xml"), "w") as f:
        f.write('<settings><z_offsets type="string">-10:0.3:5:%d</z_offsets></settings>' % nch)
    os.makedirs(os.path.join(root, fov + ".zarr"), exist_ok=True)
    return os.path.join(root, fov + ".zarr")


def loader_arm(args):
    """Decode throughput of io.FovPrefetcher (bz2 zarr chunks decoded by a pool
    of host threads into pinned memory) on one FOV of the fov3c shape read
    args.steps times."""
    import shutil
    import tempfile

    import torch

    from mermake_gb300 import io, synth
    w = WORKLOADS["fov3c"]
    Z, X, Y = w["Z"], w["X"], w["Y"]
    gain = synth.flat_gain(X, Y)
    chans = [synth.hyb_stack(Z, X, Y, w["puncta"], 1000 + 17 * c, device="cuda", gain=gain).cpu().numpy()
             for c in range(w["colours"])] + [synth.dapi_stack(Z, X, Y, 1099, device="cuda").cpu().numpy()]
    root = tempfile.mkdtemp(prefix="mm_loader_")
    t0 = time.perf_counter()
    path = write_fov_zarr(root, chans)
    t_write = time.perf_counter() - t0
    comp = sum(os.path.getsize(os.path.join(dp, f)) for dp, _, fs in os.walk(root) for f in fs)
    with io.FovPrefetcher([path] * args.warmup, prefetch=2) as pf:
        for _ in pf:
            pass
    pf = io.FovPrefetcher([path] * args.steps, prefetch=2)
    t0 = time.perf_counter()
    n = 0
    for _, im in pf:
        if isinstance(im, Exception):
            raise im
        n += 1
    wall = time.perf_counter() - t0
    pf.close()
    fov_bytes = sum(c.nbytes for c in chans)
    line = {
        "metric": "FOV decode throughput (bz2 zarr -> pinned uint16, host threads)",
        "value": n / wall,
        "unit": "FOV/s",
        "n_gpus": 1, "steps": n, "warmup": args.warmup, "ms_per_step": 1e3 * wall / n,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic fov3c channels written as the acquisition's uint8 square-root frames",
        "config": {"workload": "loader", "Z": Z, "X": X, "Y": Y, "channels": len(chans),
                   "threads": os.cpu_count(), "pinned": torch.cuda.is_available()},
        "decoded_GBps": pf.decoded_bytes / pf.decode_seconds / 1e9,
        "uint16_GBps": n * fov_bytes / wall / 1e9,
        "compressed_MB_per_fov": comp / 1e6,
        "write_s": t_write,
    }
    print(json.dumps(line), flush=True)
    shutil.rmtree(root, ignore_errors=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    if args.workload == "served":
        if rank == 0:
            served_arm(args, local)
        return
    if args.workload == "drift16":
        if rank == 0:
            drift_arm(args, local)
        return
    if args.workload == "loader":
        if rank == 0:
            import torch
            torch.cuda.set_device(local)
            loader_arm(args)
        return
    gpu_arm(args, rank, world, local)


if __name__ == "__main__":
    main()
