"""EBIV decode benchmark on GB300.

Workload (one "step" = one full decode pass over the clip): the single 1080p
stream — 1920x1080 4:2:0, 300 frames of the seeded sprite scene (24 sprites,
velocities in [-4,4] px/frame, a +40 luma flash for 3 frames every 60, noise
sigma 2 luma / 1 chroma), encoded by this repo's EBIV encoder (single-pass
mode) at q=22, gop=60, 4x3 tiles.  Synthetic data: the reference publishes no
dataset for this path (govid_gb300/workloads.py defines every clip).

Reported (one JSON line on rank 0):
  value      1080p frames/s with every packet resident in HBM before timing
             (host plans tables, kernels decode, frames land in the device
             frame pool), through the Batch API (ebivgpu_batch_*);
  bit_exact  after timing, every frame of one pass of each decode leg hashed
             (SHA-256) against the CPU oracle's decode of the same packets;
  e2e        the same clip through the public Batch API with host buffers:
             packets re-uploaded from pinned host memory and every decoded
             frame copied back to pinned host memory, inside the timed region;
  codec_api  the govid Codec contract through ebivgpu_decode: one host
             packet in, one host frame out per synchronous call;
  async_player  govid's AsyncPlayer frame source on the GPU
             (ebivgpu_source_*): frames decoded ahead and delivered to a host
             consumer in order, at decode-ahead depths 4 and 32, with and
             without WithRGBA; seek-to-first-frame time;
  roofline   algorithmic HBM bytes of a step (packets + output written once
             + one reference read per inter frame) over the step time, against
             the measured HBM copy bandwidth; per-kernel figures beside it;
  batched    64 distinct streams (24 x 640x360, 24 x 1280x720, 16 x 1920x1080,
             per-stream grid/q/gop draws, 120 frames) decoded in rounds, vs the
             same streams one stream per launch and one after another in the
             fastest single-stream mode; p50/p99 latency; bit-exact;
  serving    256 streams of 600-frame clips, Poisson requests, seeks, loops,
             HBM admission; p50/p99 request latency; bit-exact record run;
  learned_mv the learned motion-vector proposer against exhaustive search;
  cpu_baseline  the CPU oracle (the restated pure-Go decoder) on host cores.

--impl reference times the reference's CPU decoder (the oracle restatement;
Go is not available on the box) on all host cores for the same workload.  It
loads neither the GPU library nor the encoder: its clip comes from the content
cache (encoded by a child process when absent) and is demuxed by the oracle's
own container parser.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import hashlib
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

W, H, FRAMES = 1920, 1080, 300
METRIC = "EBIV 1080p frames/s (batched vs per-stream on GPU, bit-exact; p99 ms; HBM %)"

# DRAM read+write bytes per decoded frame of the 1080p clip, summed over the
# entropy, inter and intra kernels of a pipelined 32-frame-lookahead pass
# (ncu dram__bytes_read.sum + dram__bytes_write.sum over every launch of a
# 60-frame prefix decoded twice, per frame; profiles/decode_1080p_launches_traffic.md).
DRAM_BYTES_PER_FRAME = 6.22e6


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def frame_bytes(w, h):
    return w * h + 2 * ((w + 1) // 2) * ((h + 1) // 2)


def workload_name(n):
    return f"EBIV decode, 1 stream {W}x{H} {n} frames q22 gop60 tiles 4x3 (single-pass encode), 24 sprites, flashes"


def algorithmic_bytes(packets, w, h):
    """Algorithmic bytes of decoding packets: each packet read once, the
    visible output written once, one reference read per predicted sample."""
    S = frame_bytes(w, h)
    return sum(len(p) + S + (S if (p[0] & 3) == 1 else 0) for p in packets)


def sha(b) -> str:
    return hashlib.sha256(b).hexdigest()


def oracle_hashes(streams: list[list[bytes]], threads: int) -> list[list[str | None]]:
    """Per stream, per frame: SHA-256 of the oracle's packed planes (None on
    a decode error).  Streams run on a thread pool (the oracle releases the
    interpreter lock while it decodes)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import ebiv_oracle

    def one(pk):
        c = ebiv_oracle.OracleCodec(3, 1)
        out = []
        for p in pk:
            st, planes = c.decode(p)
            out.append(sha(planes) if st == 0 else None)
        return out

    with cf.ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
        return list(ex.map(one, streams))


# ---------------------------------------------------------------------------
# Clock sampling during the timed region
# ---------------------------------------------------------------------------


class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.p = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"ebiv_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in self.path.read_text().strip().splitlines() if r.strip()]
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and "Active" in r[5 + i]
                          and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# Distributed plumbing (replicas only: streams never exchange data)
# ---------------------------------------------------------------------------


def dist_init(n):
    if n <= 1 or "RANK" not in os.environ:
        return 0, 1, None
    import torch.distributed as dist

    dist.init_process_group("gloo")
    return dist.get_rank(), dist.get_world_size(), dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def flush_l2():
    import torch

    buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    buf.fill_(1)
    torch.cuda.synchronize()


def peak_hbm():
    try:
        p = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def pct(xs, q):
    s = sorted(xs)
    return s[int(q * (len(s) - 1))] if s else None


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------


def all_rounds(b, lat=None, frame_lat=None):
    """Every result of a batch until its streams are exhausted.  A pipelined
    round returns the results of the round planned b.depth calls before, so
    stop after depth + 1 empty rounds and collect the rounds in flight.  lat
    gets the wall time of each call that returned results; frame_lat gets,
    per returned frame, the wall time from the start of the call that planned
    it to the end of the call that returned it."""
    empty = 0
    starts = []
    while empty < b.depth + 1:
        t = time.perf_counter()
        starts.append(t)
        res = b.round()
        t1 = time.perf_counter()
        if lat is not None and res:
            lat.append(t1 - t)
        if frame_lat is not None and res:
            frame_lat.extend([t1 - starts[max(0, len(starts) - 1 - b.depth)]] * len(res))
        empty = empty + 1 if not res else 0
        yield from res
    yield from b.drain()


def batch_hashes(b, dims: dict) -> dict:
    """Decodes every stream of b once from the start and hashes every frame."""
    out = {}
    for sid in dims:
        b.seek(sid, 0)
    for r in all_rounds(b):
        w, h = dims[r.stream]
        out[(r.stream, r.frame_index)] = sha(b.download(r, w, h)) if r.status == 0 else None
    return out


def run_gpu(args):
    import torch

    from govid_gb300 import ebiv, workloads

    rank, world, dist = dist_init(args.gpus)
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.init()
    t0 = time.time()
    clip = workloads.load([workloads.single_1080(args.frames)], in_child=False, log=log)[0]
    log(f"[bench] content ready in {time.time() - t0:.1f}s ({len(clip)} bytes)")
    pkts = [p.data for p in ebiv.Reader(clip).packets()]
    n = len(pkts)
    alg = algorithmic_bytes(pkts, W, H)
    threads = os.cpu_count() or 1

    # ---- value: packets resident in HBM, device frame pool output ----
    depth = 0 if args.no_pipeline else args.pipeline_depth
    b = ebiv.Batch(lookahead=args.lookahead, pipeline=depth)
    sid = b.add_stream(pkts, ring=3)

    def one_pass(lat=None):
        b.seek(sid, 0)
        done = 0
        for r in all_rounds(b, lat):
            if r.status != 0:
                raise RuntimeError(f"decode failed at frame {r.frame_index}: {r.status}")
            done += 1
        return done

    for _ in range(args.warmup):
        one_pass()
    flush_l2()
    lat = []
    l0 = b.launches()
    b.timing(1)
    barrier(dist)
    torch.cuda.synchronize()
    with Clocks() as ck:
        ts = time.perf_counter()
        frames = 0
        for s in range(args.steps):
            if s:
                flush_l2()
            frames += one_pass(lat)
        torch.cuda.synchronize()
        te = time.perf_counter()
    kernel_ms, entropy_ms, recon_ms = b.timing(-1)
    launches = b.launches() - l0
    elapsed = max_over_ranks(dist, te - ts)
    value = frames * world / elapsed
    ms_per_step = elapsed * 1000 / args.steps

    # Bit-exactness of the value leg: one more pass, every frame hashed.
    want = oracle_hashes([pkts], threads)[0]
    got = batch_hashes(b, {sid: (W, H)})
    bad = [i for i in range(n) if got.get((sid, i)) != want[i]]
    if bad:
        raise RuntimeError(f"value leg: {len(bad)} frame(s) differ from the oracle, first {bad[0]}")

    # ---- e2e: the Batch API end to end.  Every step uploads the clip's
    # packets from pinned host memory (reload) and reads every decoded frame
    # back into pinned host memory (queued copies, waited for at the end).
    fb = frame_bytes(W, H)
    h2d = sum(len(p) for p in pkts)
    d2h = n * fb
    pin_pk = torch.empty(h2d, dtype=torch.uint8, pin_memory=True)
    addrs, lens, o = [], [], 0
    for p in pkts:
        pin_pk[o:o + len(p)] = torch.frombuffer(bytearray(p), dtype=torch.uint8)
        addrs.append(pin_pk.data_ptr() + o)
        lens.append(len(p))
        o += len(p)
    pin_out = torch.empty(n * fb, dtype=torch.uint8, pin_memory=True)
    eb = ebiv.Batch(lookahead=args.lookahead, pipeline=depth)
    esid = eb.add_stream(pkts, ring=3)

    def e2e_pass():
        eb.reload(esid, addrs, lens)
        k = 0
        for r in all_rounds(eb):
            if r.status != 0:
                raise RuntimeError(f"decode failed at frame {r.frame_index}: {r.status}")
            eb.download_async(r, pin_out.data_ptr() + r.frame_index * fb, fb)
            k += 1
        eb.sync()
        return k

    for _ in range(args.warmup):
        e2e_pass()
    e2e_frames = 0
    flush_l2()
    barrier(dist)
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    for s in range(args.steps):
        if s:
            flush_l2()
        e2e_frames += e2e_pass()
    torch.cuda.synchronize()
    e1 = time.perf_counter()
    e2e_elapsed = max_over_ranks(dist, e1 - e0)
    e2e = e2e_frames * world / e2e_elapsed
    host = pin_out.numpy()
    e2e_bad = [i for i in range(n) if sha(host[i * fb:(i + 1) * fb].tobytes()) != want[i]]
    if e2e_bad:
        raise RuntimeError(f"e2e leg: {len(e2e_bad)} frame(s) differ from the oracle, first {e2e_bad[0]}")

    # ---- The govid Codec contract (ebivgpu_decode): one host packet in, one
    # host frame out per synchronous call, one pass over the clip per step.
    codec = ebiv.Codec(3)
    for p in pkts[:60]:
        codec.decode(p)
    codec.flush()
    codec_frames = 0
    c0 = time.perf_counter()
    for s in range(max(1, args.steps // 4)):
        for p in pkts:
            codec.decode(p)
            codec_frames += 1
    codec_fps = codec_frames / (time.perf_counter() - c0)
    codec_bad = [i for i, p in enumerate(pkts) if sha(codec.decode(p).packed()) != want[i]]
    if codec_bad:
        raise RuntimeError(f"Codec leg: {len(codec_bad)} frame(s) differ from the oracle")
    codec.close()

    peak, peak_src = peak_hbm()
    step_gbs = alg / (ms_per_step / 1000) / 1e9
    per_step = lambda ms: ms / args.steps  # noqa: E731
    S = frame_bytes(W, H)
    inter_frames = sum(1 for p in pkts if (p[0] & 3) == 1)
    # Per stage: its algorithmic bytes over the summed time of its launches
    # (stage A reads the packets; stage B writes every output sample once and
    # reads one reference sample per predicted sample).
    kernels = {
        "entropy": {"ms_per_step": round(per_step(entropy_ms), 3), "algorithmic_bytes": h2d},
        "reconstruction": {"ms_per_step": round(per_step(recon_ms), 3),
                           "algorithmic_bytes": n * S + inter_frames * S},
    }
    for k in kernels.values():
        t = k["ms_per_step"] / 1000
        k["gbs"] = round(k["algorithmic_bytes"] / t / 1e9, 2) if t > 0 else None

    out = {
        "metric": METRIC,
        "value": round(value, 2),
        "unit": "frames/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u8",
        "data": "synthetic (seeded sprite scene encoded by this repo's EBIV encoder)",
        "config": {"workload": workload_name(n), "frames_per_step": n},
        "setup": {"packet_bytes_per_step": h2d, "l2": "flushed between steps", "lookahead_frames": args.lookahead,
                  "pipeline_depth": depth, "parallelism": f"replicas x{world}"},
        "bit_exact": True,
        "bit_exact_detail": "value, e2e and Codec legs: every frame of a pass SHA-256-equal to the CPU oracle",
        "e2e": {"value": round(e2e, 2), "unit": "frames/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "api": "Batch API: packets reloaded from pinned host memory, every frame copied to pinned host memory"},
        "codec_api": {"frames_per_s": round(codec_fps, 2), "api": "ebivgpu_decode (govid Codec.Decode): one host "
                      "packet in, one host frame out, synchronous"},
        "latency_ms": {"p50": round(1000 * statistics.median(lat), 3) if lat else None,
                       "p99": round(1000 * pct(lat, 0.99), 3) if lat else None},
        "roofline": {"bound": "hbm", "achieved": round(step_gbs, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(step_gbs / peak, 4),
                     "traffic": int(DRAM_BYTES_PER_FRAME * n),
                     "algorithmic_bytes": int(alg),
                     "kernel": "the whole decode step (entropy, inter and intra kernels overlap); algorithmic "
                               "bytes of a step over ms_per_step",
                     "peak_source": peak_src, "kernels": kernels,
                     "kernel_time_sum_ms_per_step": round(per_step(kernel_ms), 3)},
        "gpu_launches": launches,
    }
    if rank == 0:
        if not args.no_batched:
            out["batched"] = run_batched(args)
        if not args.no_serve:
            out["serving"] = run_serve(args)
        if not args.no_mv:
            from govid_gb300 import eval_mvnet

            r = eval_mvnet.compare(1920, 1080, nframes=args.mv_frames, qp=22, log=None)
            r["note"] = "encoder on the host cores; the proposer's net runs on this GPU"
            out["learned_mv"] = r
        if not args.no_extras:
            out["rgba"] = run_rgba(pkts, want)
            out["async_player"] = run_async_source(clip, pkts, want)
            out["ingest"] = run_ingest(clip, pkts, want)
            out["altref"] = run_altref()
            out["block_analysis"] = run_analysis()
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(pkts, args.cpu_seconds)
        out["clocks"] = ck.summary()
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_rgba(pkts, want):
    """WithRGBA (source.go:61-74): the Codec contract with the RGBA pass in
    each decode round (kRGBA on the device frame, pooled pinned output),
    against the same contract without it and the CPU conversion
    (frame.go:8-67, the oracle's C++ restatement) per 1080p frame."""
    import numpy as np

    from govid_gb300 import ebiv

    sys.path.insert(0, str(ROOT / "oracle"))
    import ebiv_oracle

    c = ebiv.Codec(3)
    c.with_rgba(True)
    for p in pkts[:30]:
        c.decode(p)
    c.flush()
    t0 = time.perf_counter()
    for p in pkts:
        c.decode(p)
    fps = len(pkts) / (time.perf_counter() - t0)
    # bit-exactness of the pooled RGBA on a few frames of a fresh pass
    c.flush()
    bad = 0
    for i, p in enumerate(pkts[:8]):
        f = c.decode(p)
        ref = np.frombuffer(ebiv_oracle.rgba(f.packed(), W, H), np.uint8).reshape(H, W, 4)
        bad += int(not (c.pooled_rgba(f) == ref).all())
    c.close()
    if bad:
        raise RuntimeError(f"rgba: {bad} frame(s) differ from the oracle")
    f0 = ebiv_oracle.decode_all(pkts[:1])[0][1]
    t0 = time.perf_counter()
    reps = 20
    for _ in range(reps):
        ebiv_oracle.rgba(f0, W, H)
    cpu_ms = (time.perf_counter() - t0) * 1000 / reps
    return {"codec_with_rgba_frames_per_s": round(fps, 2), "bit_exact_frames_checked": 8,
            "cpu_rgba_ms_per_1080p_frame": round(cpu_ms, 3),
            "note": "CPU: the oracle's C++ restatement of convertYCbCr420ToRGBA, one thread"}


def run_async_source(clip, pkts, want):
    """govid's AsyncPlayer frame source on the GPU (ebivgpu_source_*): a
    consumer taking every frame of the clip into host memory through next()
    and releasing it, at the decode-ahead depth of govid's Ebitengine example
    (4, with and without WithRGBA) and at 32; plus the time from Seek to the
    first frame at 16 key frames.  Every frame of one pass is hashed."""
    import numpy as np

    from govid_gb300 import ebiv

    n = len(pkts)
    rd = ebiv.Reader(clip)
    out = {}
    for depth, rgba in ((4, False), (4, True), (32, False)):
        src = ebiv.AsyncSource(clip, depth=depth, rgba=rgba)
        for rep in range(3):  # two warm passes, then the timed one
            src.seek(0)
            t0 = time.perf_counter()
            k = 0
            for _ in range(n):
                f = src.next()
                k += 1
                src.release(f)
            dt = time.perf_counter() - t0
        out[f"depth{depth}{'_rgba' if rgba else ''}_frames_per_s"] = round(k / dt, 2)
        if not rgba:
            src.seek(0)
            got = []
            for _ in range(n):
                f = src.next()
                got.append(sha(f.packed()))
                src.release(f)
            if got != want:
                raise RuntimeError(f"async source depth {depth}: frames differ from the oracle")
        if depth == 4 and not rgba:
            keys = [i for i, p in enumerate(pkts) if (p[0] & 3) == 0]
            lat = []
            for j in range(16):
                t = rd.frame_time(keys[j % len(keys)] + 1)
                t0 = time.perf_counter()
                src.seek(t)
                f = src.next()
                lat.append(time.perf_counter() - t0)
                src.release(f)
            out["seek_to_first_frame_ms"] = {"p50": round(1000 * statistics.median(lat), 3),
                                             "max": round(1000 * max(lat), 3)}
        src.destroy()
    out["bit_exact"] = True
    out["note"] = ("frames delivered to a host consumer in order, each copied to pinned host memory "
                   "(and converted to RGBA on the GPU with WithRGBA)")
    return out


def run_ingest(clip, pkts, want):
    """Container ingest on the GPU: index build and seeks on the device over
    the pinned container, and a batch stream decoding in place from it,
    bit-exact, against the same stream with its packets copied to HBM."""
    from govid_gb300 import ebiv

    t0 = time.perf_counter()
    dc = ebiv.DeviceContainer(clip)
    open_ms = (time.perf_counter() - t0) * 1000
    r = ebiv.Reader(clip)
    t0 = time.perf_counter()
    seeks = [k * 997_000_000 // 7 for k in range(64)]
    for t in seeks:
        assert dc.seek(t)[1] == r.seek(t)
    seek_us = (time.perf_counter() - t0) * 1e6 / len(seeks)
    out = {"open_ms": round(open_ms, 3), "seek_us": round(seek_us, 2), "frames": dc.frame_count}
    for name, add in (("in_place", lambda b: b.add_container(dc)), ("copied", lambda b: b.add_stream(pkts))):
        b = ebiv.Batch(lookahead=32, pipeline=3)
        sid = add(b)
        for rep in range(3):
            b.seek(sid, 0)
            t0 = time.perf_counter()
            n = sum(1 for x in all_rounds(b) if x.status == 0)
            dt = time.perf_counter() - t0
        out[f"{name}_frames_per_s"] = round(n / dt, 2)
        got = batch_hashes(b, {sid: (W, H)})
        if [got[(sid, i)] for i in range(len(pkts))] != want:
            raise RuntimeError(f"ingest {name}: frames differ from the oracle")
        b.close()
    out["bit_exact"] = True
    return out


def run_altref():
    """The alt-ref temporal filter ((*Encoder).buildAltRef,
    ebiv/encoder.go:326-407) on the GPU over 16 1080p frames: kernel time and
    HBM rate (16 frames read, one written), bit-exact against the numpy
    restatement."""
    from govid_gb300 import ebiv

    sys.path.insert(0, str(ROOT / "oracle"))
    import altref_ref

    sc = ebiv.Scene(ebiv.SceneSpec(width=W, height=H, seed=9, sprites=24, noise_y16=16, noise_c16=8))
    frames = [sc.render(i) for i in range(16)]
    a = ebiv.AltRef()
    got = a.build(frames, W, H, 16)
    t0 = time.perf_counter()
    want = altref_ref.build_altref(frames, W, H, 16)
    cpu_s = time.perf_counter() - t0
    if got != want:
        raise RuntimeError("altref: GPU filter differs from the oracle")
    ms = a.time(16, 20)
    S = frame_bytes(W, H)
    gbs = 17 * S / (ms / 1000) / 1e9
    peak, _ = peak_hbm()
    return {"frames": 16, "kernel_ms": round(ms, 4), "hbm_gbs": round(gbs, 2), "hbm_frac": round(gbs / peak, 4),
            "accepted_blocks": a.accepted, "bit_exact": True, "oracle_numpy_s": round(cpu_s, 3)}


def run_analysis():
    """forwardDCT + satd (ebiv/transform.go:44-119) of 1M 8x8 residual
    blocks on the GPU, kernel time, bit-exact on a sample against the numpy
    restatement."""
    import numpy as np

    from govid_gb300 import ebiv

    sys.path.insert(0, str(ROOT / "oracle"))
    import transform_ref

    rng = np.random.default_rng(1)
    blocks = rng.integers(-255, 256, size=(1 << 20, 8, 8), dtype=np.int64).astype(np.int32)
    a = ebiv.BlockAnalysis()
    co, sa = a.fdct_satd(blocks)
    co, sa = a.fdct_satd(blocks)
    ms = a.kernel_ms
    k = 4096
    if not ((co[:k] == transform_ref.forward_dct(blocks[:k], 8)).all() and
            (sa[:k] == transform_ref.satd(blocks[:k], 8)).all()):
        raise RuntimeError("block analysis differs from the oracle")
    byts = blocks.nbytes * 2 + sa.nbytes
    peak, _ = peak_hbm()
    return {"blocks": len(blocks), "n": 8, "kernel_ms": round(ms, 4), "blocks_per_s": round(len(blocks) / ms * 1e3),
            "hbm_gbs": round(byts / (ms / 1000) / 1e9, 2), "hbm_frac": round(byts / (ms / 1000) / 1e9 / peak, 4),
            "bit_exact_sample": k}


def run_batched(args):
    """64 distinct mixed streams in rounds vs the same streams one stream per
    launch, at each lookahead of --mix-lookahead (the first is the headline:
    the latency-bounded configuration; the last the throughput one)."""
    import torch

    from govid_gb300 import ebiv, workloads

    t0 = time.time()
    clips = workloads.mix(args.mix_frames)
    conts = workloads.load(clips, in_child=False, log=log)
    log(f"[bench] mix content ready in {time.time() - t0:.1f}s")
    pkts = [[p.data for p in ebiv.Reader(c).packets()] for c in conts]
    dims = [(c.w, c.h) for c in clips]
    alg = sum(algorithmic_bytes(pk, w, h) for pk, (w, h) in zip(pkts, dims))
    totals = sum(len(pk) for pk in pkts)
    px = sum(len(pk) * w * h for pk, (w, h) in zip(pkts, dims))
    eq1080 = px / (W * H)  # frames of the mix in 1080p-frame units
    peak, _ = peak_hbm()
    depth = 0 if args.no_pipeline else args.mix_depth

    def one(lookahead, dep=depth, groups=4, warps=0):
        b = ebiv.Batch(lookahead=lookahead, pipeline=dep)
        b.set_tuning(groups, warps)
        ids = [b.add_stream(pk, ring=3) for pk in pkts]
        for sid in ids:  # warm-up round
            b.seek(sid, 0)
        b.round()
        b.drain()
        for sid in ids:
            b.seek(sid, 0)
        flush_l2()
        lat, flat = [], []
        torch.cuda.synchronize()
        b.timing(1)
        ts = time.perf_counter()
        frames = 0
        for r in all_rounds(b, lat, flat):
            frames += 1
            if r.status != 0:
                raise RuntimeError(f"batched decode failed: {r}")
        torch.cuda.synchronize()
        te = time.perf_counter()
        kernel_ms, _, _ = b.timing(-1)
        fps = frames / (te - ts)
        gbs = alg / (te - ts) / 1e9
        res = {"lookahead_frames": lookahead, "pipeline_depth": dep, "entropy_groups": groups, "intra_warps": warps,
               "frames": frames, "frames_per_s": round(fps, 2),
               "frames_1080p_equiv_per_s": round(eq1080 / (te - ts), 2),
               "round_latency_ms": {"p50": round(1000 * statistics.median(lat), 3),
                                    "p99": round(1000 * pct(lat, 0.99), 3)},
               "frame_latency_ms": {"p50": round(1000 * statistics.median(flat), 3),
                                    "p99": round(1000 * pct(flat, 0.99), 3)},
               "hbm_gbs": round(gbs, 2), "hbm_frac": round(gbs / peak, 4),
               "kernel_time_sum_ms": round(kernel_ms, 3)}
        return res, b, ids

    runs = []
    check_b = None
    for k in str(args.mix_lookahead).split(","):
        res, b, ids = one(int(k))
        runs.append(res)
        if check_b is None:
            check_b, check_ids = b, ids
        else:
            b.close()
    # The autotuner's choice (throughput objective, tried on 16-frame prefixes).
    tuned = None
    if not args.no_autotune:
        from govid_gb300 import autotune

        t0 = time.time()
        tn = autotune.tune(pkts, frames=16, objective="throughput")
        c = tn["choice"]
        res, b, _ = one(c["lookahead"], c["pipeline_depth"], c["entropy_groups"], c["intra_warps"])
        b.close()
        tuned = {"choice": {k: c[k] for k in ("lookahead", "pipeline_depth", "entropy_groups", "intra_warps")},
                 "tuning_s": round(time.time() - t0, 1), "trials": len(tn["trials"]), "run": res,
                 "vs_hand_picked_throughput_config": round(res["frames_per_s"] / runs[-1]["frames_per_s"], 3)}
    # Bit-exactness of the batched decode: every frame of every stream.
    want = oracle_hashes(pkts, os.cpu_count() or 1)
    got = batch_hashes(check_b, {sid: dims[i] for i, sid in enumerate(check_ids)})
    nbad = sum(1 for i, sid in enumerate(check_ids) for f in range(len(pkts[i])) if got.get((sid, f)) != want[i][f])
    check_b.close()
    if nbad:
        raise RuntimeError(f"batched leg: {nbad} frame(s) differ from the oracle")

    # One stream per launch: each stream decoded alone, one frame per
    # synchronous round (one set of launches per frame).
    single_b = ebiv.Batch(lookahead=1)
    single_ids = [single_b.add_stream(pk, ring=3) for pk in pkts]
    flush_l2()
    torch.cuda.synchronize()
    s0 = time.perf_counter()
    single = 0
    for sid in single_ids:
        while True:
            res = single_b.round([sid])
            if not res:
                break
            single += len(res)
    torch.cuda.synchronize()
    per_launch_s = time.perf_counter() - s0
    single_b.close()
    # The same streams one after another in the fastest single-stream mode
    # (32-frame lookahead, pipeline depth 3), as the value leg decodes.
    best_b = ebiv.Batch(lookahead=args.lookahead, pipeline=args.pipeline_depth)
    best_ids = [best_b.add_stream(pk, ring=3) for pk in pkts]
    flush_l2()
    torch.cuda.synchronize()
    b0 = time.perf_counter()
    best = 0
    for sid in best_ids:
        best_b.seek(sid, 0)
    for sid in best_ids:
        for r in best_b_rounds(best_b, sid):
            best += 1
    torch.cuda.synchronize()
    best_s = time.perf_counter() - b0
    best_b.close()
    per_launch_fps = single / per_launch_s
    best_fps = best / best_s
    for r in runs:
        r["speedup_vs_one_stream_per_launch"] = round(r["frames_per_s"] / per_launch_fps, 3)
        r["speedup_vs_streams_in_turn_best_mode"] = round(r["frames_per_s"] / best_fps, 3)
    out = {"streams": len(clips), "distinct_bitstreams": len({sha(c) for c in conts}),
           "stream_draws": [c.describe() for c in clips], "pipeline_depth": depth,
           "frames_per_stream": args.mix_frames, "frames_1080p_equiv": round(eq1080, 1),
           "bit_exact": True, "bit_exact_frames": sum(len(p) for p in pkts),
           "one_stream_per_launch": {"frames_per_s": round(per_launch_fps, 2),
                                     "frames_1080p_equiv_per_s": round(eq1080 / per_launch_s, 2),
                                     "how": "each stream alone, one frame per synchronous round"},
           "streams_in_turn_best_mode": {"frames_per_s": round(best_fps, 2),
                                         "frames_1080p_equiv_per_s": round(eq1080 / best_s, 2),
                                         "how": f"each stream alone, lookahead {args.lookahead}, pipeline depth "
                                                f"{args.pipeline_depth}"}}
    out.update(runs[0])
    if len(runs) > 1:
        out["throughput_config"] = runs[-1]
    if tuned:
        tuned["run"]["speedup_vs_one_stream_per_launch"] = round(tuned["run"]["frames_per_s"] / per_launch_fps, 3)
        out["autotuned"] = tuned
    out["packet_bytes"] = totals
    return out


def best_b_rounds(b, sid):
    """All results of one stream of a pipelined batch, decoded alone."""
    empty = 0
    while empty < b.depth + 1:
        res = b.round([sid])
        empty = empty + 1 if not res else 0
        yield from res
    yield from b.drain()


def run_serve(args):
    """256 streams with per-frame requests arriving as Poisson processes at
    30 or 60 fps, 5 % seeks, 10 % looping streams, HBM admission cap 120 GB;
    continuous batching; per-request latency from arrival to delivery.  A
    second, shorter run in record mode hashes every delivered frame and checks
    it against the oracle's decode of that stream alone."""
    import random

    from govid_gb300 import ebiv, workloads

    clips = workloads.serve(args.serve_frames)
    conts = workloads.load(clips, in_child=False, log=log)
    base = [[p.data for p in ebiv.Reader(c).packets()] for c in conts]

    def server(record, seconds, key_cache=None):
        rng = random.Random(args.serve_seed)
        srv = ebiv.Server(duration_s=seconds, frames_per_stream=args.serve_frames, seek_prob=0.05,
                          seed=args.serve_seed, hbm_budget_bytes=120 << 30,
                          max_frames_per_round=args.serve_max_frames, ring=3, key_lane=args.serve_key_lanes,
                          start_spread_s=1.0, record=record, decode_ahead=args.serve_ahead,
                          key_cache=args.serve_key_cache if key_cache is None else key_cache)
        counts, which = {}, []
        for i in range(args.serve_streams):
            k = i % len(clips)
            srv.add_stream(base[k], fps=rng.choice([30, 60]), loop=rng.random() < 0.10)
            which.append(k)
            key = f"{clips[k].w}x{clips[k].h}"
            counts[key] = counts.get(key, 0) + 1
        return srv, counts, which

    # The streams without preparation first: their first requests find empty
    # decode-ahead buffers and their long key frames undecoded.
    usrv, _, _ = server(False, args.serve_seconds, key_cache=1)
    ust = usrv.run()
    del usrv
    srv, counts, _ = server(False, args.serve_seconds)
    st = srv.run()
    out = {
        "streams": args.serve_streams, "resolutions": counts, "clip_frames": args.serve_frames,
        "distinct_clips": len(clips), "clip_draws": [c.describe() for c in clips],
        "request_window_s": args.serve_seconds, "admitted_total": st["admitted_total"],
        "admitted_peak": st["admitted_peak"], "hbm_cap_gb": 120, "peak_state_gb": round(st["peak_bytes"] / 2**30, 3),
        "requests": st["requests"], "frames": st["frames"], "errors": st["errors"], "seeks": st["seeks"],
        "loops": st["loops"], "rounds": st["rounds"], "frames_per_s": round(st["frames_per_s"], 2),
        "latency_ms": {"p50": round(st["latency_p50_ms"], 3), "p99": round(st["latency_p99_ms"], 3),
                       "max": round(st["latency_max_ms"], 3), "mean": round(st["latency_mean_ms"], 3)},
        "seek_latency_ms": {"p50": round(st["seek_latency_p50_ms"], 3), "p99": round(st["seek_latency_p99_ms"], 3)},
        "ready_at_arrival_frac": round(st["ready_at_arrival"] / max(1, st["frames"]), 4),
        "unserved_past_clip_end": st["unserved"],
        "frames_per_round": args.serve_max_frames, "decode_ahead": args.serve_ahead,
        "elapsed_s": round(st["elapsed_s"], 3),
        "decode_thread": {"main_rounds": st["main_rounds"], "side_rounds": st["side_rounds"],
                          "main_round_frames": st["main_frames"], "main_round_s": round(st["main_round_s"], 3),
                          "idle_s": round(st["idle_s"], 3), "plan_s": round(st["plan_s"], 3),
                          "collect_s": round(st["collect_s"], 3), "kernel_ms": round(st["kernel_ms"], 1),
                          "entropy_ms": round(st["entropy_ms"], 1), "recon_ms": round(st["recon_ms"], 1)},
        "side_lanes": args.serve_key_lanes, "key_cache": args.serve_key_cache, "key_installs": st["key_installs"],
        "seek_shortcuts": st["seek_shortcuts"], "follow_rounds": st["follow_rounds"],
        "prepare_s": round(st["prepare_s"], 3),
        "unprepared": {"key_cache": 1, "requests": ust["requests"], "frames": ust["frames"],
                       "frames_per_s": round(ust["frames_per_s"], 2), "elapsed_s": round(ust["elapsed_s"], 3),
                       "latency_ms": {"p50": round(ust["latency_p50_ms"], 3), "p99": round(ust["latency_p99_ms"], 3),
                                      "max": round(ust["latency_max_ms"], 3)},
                       "seek_latency_ms": {"p50": round(ust["seek_latency_p50_ms"], 3),
                                           "p99": round(ust["seek_latency_p99_ms"], 3)}},
        "start_spread_s": 1.0, "key_frames": st["key_frames"],
    }
    del srv
    # Record run: every delivered frame's FNV-1a against the oracle's.
    rsrv, _, which = server(True, args.serve_check_seconds)
    rsrv.run()
    hashes = rsrv.frame_hashes()
    del rsrv
    need = sorted({which[s] for s, _, _ in hashes})
    sys.path.insert(0, str(ROOT / "oracle"))
    import ebiv_oracle

    def oracle_fnv(k):
        c = ebiv_oracle.OracleCodec(3, 1)
        return [ebiv.frame_hash(pl) if st == 0 else None for st, pl in (c.decode(p) for p in base[k])]

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        ref = dict(zip(need, ex.map(oracle_fnv, need)))
    bad = sum(1 for s, f, h in hashes if ref[which[s]][f] != h)
    if bad:
        raise RuntimeError(f"serving: {bad} delivered frame(s) differ from the oracle")
    out["bit_exact"] = True
    out["bit_exact_check"] = {"delivered_frames_hashed": len(hashes), "request_window_s": args.serve_check_seconds}
    return out


# ---------------------------------------------------------------------------
# CPU baseline / reference arm (the oracle: the restated pure-Go decoder)
# ---------------------------------------------------------------------------


def cpu_baseline(pkts, seconds: float):
    sys.path.insert(0, str(ROOT / "oracle"))
    import ebiv_oracle

    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    done = 0
    reps = 0
    while time.perf_counter() - t0 < seconds or reps == 0:
        res = ebiv_oracle.decode_all(pkts, threads=threads)
        done += sum(1 for s, _ in res if s == 0)
        reps += 1
    dt = time.perf_counter() - t0
    return {"value": round(done / dt, 2), "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": f"{reps} pass(es) over the {len(pkts)}-frame 1080p clip, tiles on a {threads}-thread pool"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from govid_gb300 import workloads  # content cache only: loads no native code

    clip = workloads.load([workloads.single_1080(args.frames)], in_child=True)[0]
    sys.path.insert(0, str(ROOT / "oracle"))
    import ebiv_container
    import ebiv_oracle

    pkts = ebiv_container.packets(clip)
    threads = os.cpu_count() or 1
    for _ in range(max(1, min(args.warmup, 1))):
        ebiv_oracle.decode_all(pkts[:30], threads=threads)
    t0 = time.perf_counter()
    frames = 0
    for _ in range(args.steps):
        res = ebiv_oracle.decode_all(pkts, threads=threads)
        frames += sum(1 for s, _ in res if s == 0)
    dt = time.perf_counter() - t0
    v = frames / dt
    out = {
        "impl": "reference",
        "metric": METRIC,
        "value": round(v, 2), "unit": "frames/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * dt / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded sprite scene encoded by this repo's EBIV encoder)",
        "config": {"workload": workload_name(len(pkts)), "frames_per_step": len(pkts)},
        "cpu_baseline": {"value": round(v, 2), "unit": "frames/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full pass(es) of the clip, tiles on a {threads}-thread pool"},
        "e2e": {"value": round(v, 2), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--frames", type=int, default=FRAMES)
    ap.add_argument("--mix-frames", type=int, default=120)
    ap.add_argument("--lookahead", type=int, default=32)
    ap.add_argument("--mix-lookahead", default="1,4", help="comma list: headline (latency-bounded) first")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-pipeline", action="store_true", help="synchronous rounds (no entropy/recon overlap)")
    ap.add_argument("--mix-depth", type=int, default=2, help="pipeline depth of the 64-stream rounds")
    ap.add_argument("--pipeline-depth", type=int, default=3,
                    help="rounds planned ahead of the one reconstructing (single-stream legs)")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-mv", action="store_true")
    ap.add_argument("--mv-frames", type=int, default=120)
    ap.add_argument("--serve-streams", type=int, default=256)
    ap.add_argument("--serve-frames", type=int, default=600)
    ap.add_argument("--serve-seconds", type=float, default=4.0)
    ap.add_argument("--serve-check-seconds", type=float, default=1.5)
    ap.add_argument("--serve-max-frames", type=int, default=4, help="frames of one stream per serving round")
    ap.add_argument("--serve-ahead", type=int, default=6, help="frames decoded ahead of each stream's requests")
    ap.add_argument("--serve-key-lanes", type=int, default=3, help="side lanes for key frames with long chains")
    ap.add_argument("--serve-key-cache", type=int, default=3,
                    help="1: streams with long key frames reinstall key frames they decoded before; 2: and decode "
                         "them all at admission, and the streams admitted at start fill their decode-ahead, "
                         "before the request clock starts (reported as prepare_s); 3: as 2 for every stream")
    ap.add_argument("--serve-seed", type=int, default=4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the RGBA, ingest, alt-ref and analysis legs")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
