"""Render-throughput benchmark of the nerf-tf2 render path on GB300.

One step = one full 800x800 pinhole frame (640,000 rays) rendered
hierarchically in 4096-ray chunks with 64 coarse + 128 fine samples per ray
(the reference's render loop, nerf/main/render.py:79-93 with
base_dataset.py:797-861), random-init coarse and fine networks, synthetic
camera on the radius-4 sphere.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--path bf16|fp32] [--proposal 0|1]
    python bench.py --impl reference ...   # the reference algorithm on host cores

Prints one JSON line (rank 0). `value` is whole-job rays/s of the BF16 +
learned-proposal path (proposal-gated: the proposal's weights decide which
coarse samples the NeRF MLP evaluates) with rays resident in HBM; `e2e` is
the same through NeRF.render with the rays in pinned host memory and the
rgb/depth/acc maps copied back every step. `plain_fp32` is the plain FP32
coarse+fine path on the same frame, `quality` the PSNR of both against a
64+512-sample render; `proposal.replace` reports the proposal used as the
fine sampler's PDF in place of the coarse pass.
"""
import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "rays/s coarse+fine render, BF16+proposal vs plain FP32, at ≤0.1 dB PSNR gap"
H = W = 800
FOCAL = 1111.111
CHUNK = 4096
SC, SF = 64, 128
FLOP_PER_SAMPLE = 1186816          # 2 x 593,408 MAC of the 8x256 MLP + heads
L2_FLUSH_BYTES = 512 << 20         # > 129 MB L2
SCENE_SEED = 21
SCENE_MAX_FREQ_LOG2 = 6  # scene band-limited to the proposal's encoding (L=6)
WORKLOAD = ("800x800 pinhole frame (focal 1111.111) from a random camera on the radius-4 sphere, "
            "4096-ray chunks, 64 stratified + 128 fine samples; scene = one random-init 8x256 network "
            "(sigma head x4, bias -0.5, xyz encoding cut above 2^5 pi) as coarse and fine")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--path", default="bf16", choices=["bf16", "fp8", "fp32"])
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--kernel", default=None, choices=["mlp", "train", "chain"],
                    help="mlp: the MLP kernel alone at the fine-pass launch shape; train: training steps; "
                         "chain: the gated render of --chunks 4096-ray chunks (for ncu captures)")
    ap.add_argument("--chunks", type=int, default=4)
    ap.add_argument("--batch", type=int, default=4096, help="rays per training step of --kernel train")
    ap.add_argument("--rows", type=int, default=CHUNK * (SC + SF))
    ap.add_argument("--proposal", type=int, default=1, help="1: BF16 + learned proposal (headline)")
    ap.add_argument("--proposal-mode", default="gate", choices=["gate", "replace"])
    ap.add_argument("--gate-tau", type=float, default=1e-4)
    ap.add_argument("--streams", type=int, default=3,
                    help="streams the render's chunks alternate over (NeRF.render(streams=)) and "
                         "the training backward runs on (NeRF.backward_streams)")
    ap.add_argument("--gate-fine-draws", type=int, default=1,
                    help="1: the gate also skips fine draws in coarse bins the proposal calls empty")
    ap.add_argument("--proposal-steps", type=int, default=2000)
    ap.add_argument("--train-steps", type=int, default=3)
    ap.add_argument("--train-tile", type=int, default=1024,
                    help="rays per recompute tile of the training backward's tiled line (0: keep the forward's tape)")
    ap.add_argument("--sweep", type=int, default=1, help="1: FP32/BF16/FP8 sweep at 65536 rays x 256")
    ap.add_argument("--glorot-scene", type=int, default=1,
                    help="1: the gated path also on a plain Glorot-initialised scene with its own proposal")
    return ap.parse_args()


def kernel_only(args):
    """The MLP kernel alone, `--steps` launches on `--rows` rows (the fine pass
    of one 4096-ray chunk by default). Prints the median launch time."""
    import torch
    ng = importlib.import_module("nerf-tf2_gb300")
    dev = torch.device("cuda", 0)
    torch.manual_seed(0)
    xyz = torch.rand(args.rows, 3, device=dev) * 4 - 2
    dirs = torch.nn.functional.normalize(torch.randn(args.rows, 3, device=dev), dim=1)
    mlp = ng.get_coarse_or_fine_model("fine", seed=1, precision=args.path)
    for _ in range(args.warmup):
        mlp((xyz, dirs))
    ts = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        mlp((xyz, dirs))
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    mlp.check_device_errors()
    ms = statistics.median(ts)
    print(json.dumps({"kernel": f"mlp_{args.path}", "rows": args.rows, "launch_ms": ms,
                      "tflops": args.rows * FLOP_PER_SAMPLE / ms / 1e9}), flush=True)


def train_only(args):
    """`--steps` training steps (4096 rays of the benchmark scene, precision
    `--path`) after `--warmup` untimed ones. Prints the median step time."""
    import torch
    ng = importlib.import_module("nerf-tf2_gb300")
    dev = torch.device("cuda", 0)
    params = ng.make_params(N_coarse=SC, N_fine=SF)
    blob = ng.synthetic.sparse_scene_blob(SCENE_SEED, max_freq_log2=SCENE_MAX_FREQ_LOG2)
    teacher = ng.NeRF(params, precision="fp32", coarse_params=blob, fine_params=blob)
    batch = [torch.from_numpy(x[:args.batch]).to(dev)
             for x in ng.synthetic.training_rays(500, 4, (args.batch + 3) // 4)]
    target = teacher.render(*batch, seed=3)["rgb"]
    student = ng.NeRF(params, precision=args.path, seed=60)
    student.backward_streams = args.streams
    tile = args.train_tile or None
    for _ in range(args.warmup):
        student.train_step((tuple(batch), (target,)), tile_rays=tile)
    ts = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        student.train_step((tuple(batch), (target,)), tile_rays=tile)
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    student.coarse_model.check_device_errors()
    print(json.dumps({"kernel": f"train_{args.path}", "batch_rays": args.batch, "tile_rays": tile,
                      "step_ms": statistics.median(ts)}), flush=True)


def chain_only(args):
    """The gated render (untrained proposal) of the benchmark frame's first
    `--chunks` 4096-ray chunks, `--warmup` + `--steps` times: the ray
    kernels of one chunk at their render shapes, for ncu captures. Prints the
    median step time."""
    import torch
    ng = importlib.import_module("nerf-tf2_gb300")
    dev = torch.device("cuda", 0)
    params = ng.make_params(N_coarse=SC, N_fine=SF)
    blob = ng.synthetic.sparse_scene_blob(SCENE_SEED, max_freq_log2=SCENE_MAX_FREQ_LOG2)
    nerf = ng.NeRF(params, precision=args.path, coarse_params=blob, fine_params=blob)
    prop = ng.ProposalNetwork(seed=7)
    n = CHUNK * args.chunks
    rays = [torch.from_numpy(x[:n]).to(dev) for x in ng.synthetic.frame_rays(0, H, W, FOCAL)]
    ts = []
    for i in range(args.warmup + args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        nerf.render(*rays, chunk=CHUNK, streams=args.streams,
                    seed=i, proposal=prop, proposal_mode="gate", gate_tau=args.gate_tau,
                    gate_fine_draws=bool(args.gate_fine_draws))
        e1.record()
        torch.cuda.synchronize()
        if i >= args.warmup:
            ts.append(e0.elapsed_time(e1))
    nerf.coarse_model.check_device_errors()
    print(json.dumps({"kernel": "chain", "rays": n, "step_ms": statistics.median(ts)}), flush=True)


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def rank_frame_seed(rank):
    """Weak scaling: rank r renders its own frame, from camera seed r (rays
    are independent; no data-path collective)."""
    return rank


def max_over_ranks(total_ms, world, device):
    """The slowest rank's summed step time (all_reduce MAX; identity at 1)."""
    import torch
    import torch.distributed as tdist
    t = torch.tensor([float(total_ms)], device=device, dtype=torch.float64)
    if world > 1:
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, units_per_rank, ms_per_step):
    """Units per second over all ranks: every rank's units / the slowest rank's step time."""
    return world * units_per_rank / (ms_per_step / 1000.0)


# ---------------------------------------------------------------------------
# CPU side: the oracle restatement of the reference algorithm
# ---------------------------------------------------------------------------
def cpu_render_rate(ng, frame, seconds, max_rays=4096, block=128):
    """Times the oracle's FP32 hierarchical render of the benchmark scene on
    consecutive 128-ray blocks of the frame until `seconds` elapse. Returns
    (rays/s, rays)."""
    oracle = importlib.import_module("oracle")
    o, d, n, f = frame
    p = ng.make_params()
    pc = pf = oracle.unpack_params(ng.synthetic.sparse_scene_blob(SCENE_SEED, max_freq_log2=SCENE_MAX_FREQ_LOG2))
    rng = np.random.default_rng(0)
    done, t0 = 0, time.perf_counter()
    while done < max_rays and (time.perf_counter() - t0) < seconds:
        s = slice(done, done + block)
        uc = rng.random((block, SC), dtype=np.float32)
        uf = rng.random((block, SF), dtype=np.float32)
        oracle.nerf_forward(p, pc, pf, o[s], d[s], n[s], f[s], uc, uf, np.float32)
        done += block
    return done / (time.perf_counter() - t0), done


def reference_arm(args):
    rank, _, world = dist_env()
    if rank != 0:
        return
    ng = importlib.import_module("nerf-tf2_gb300")
    frame = ng.synthetic.frame_rays(0, H, W, FOCAL)
    cores = os.cpu_count()
    per_step = 256
    for _ in range(args.warmup):
        cpu_render_rate(ng, frame, 1e9, max_rays=per_step)
    rates = [cpu_render_rate(ng, frame, 1e9, max_rays=per_step)[0] for _ in range(args.steps)]
    rate = statistics.mean(rates)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "rays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * per_step / rate,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_rays_per_step": per_step,
                   "path": "plain FP32 hierarchical (the reference's algorithm)"},
        "cpu_baseline": {"value": rate, "unit": "rays/s", "cores": cores, "kind": "port",
                         "sample": f"{per_step} rays of the frame per step; numpy FP32 restatement "
                                   "(TensorFlow 2.6 is not installable here), OpenBLAS on all cores"},
        "e2e": {"value": rate, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Errors against the FP64 oracle (untimed): a fixed subset of rays rendered
# on the GPU with explicit uniforms, and the same rays through the oracle's
# FP64 chain with the same uniforms.
# ---------------------------------------------------------------------------
def fp64_subset(rays, n=256, seed=123, n_fine=SF):
    """n rays spread over the frame (every R//n-th) and their uniforms."""
    import torch
    R = rays[0].shape[0]
    idx = torch.arange(0, R, max(1, R // n), device=rays[0].device)[:n]
    sub = [x[idx].contiguous() for x in rays]
    rng = np.random.default_rng(seed)
    uc = rng.random((len(idx), SC), dtype=np.float32)
    uf = rng.random((len(idx), n_fine), dtype=np.float32)
    return sub, uc, uf


def fp64_errors(got_rgb, want_rgb):
    g = np.asarray(got_rgb, np.float64)
    w = np.asarray(want_rgb, np.float64)
    mse = float(np.mean((g - w) ** 2))
    return {"max_abs_rgb": float(np.abs(g - w).max()), "mean_abs_rgb": float(np.abs(g - w).mean()),
            "psnr_db": float(-10.0 * np.log10(max(mse, 1e-30)))}


def config1(ng, dev, blob_seed=(1, 2), steps=20, warmup=3):
    """The coarse pass alone on 1,024 sphere rays (64 stratified samples,
    Glorot-initialised network): rays/s per precision (CUDA events over
    `steps` passes, inputs resident) and errors against the FP64 oracle's
    coarse pass on all 1,024 rays."""
    import torch
    oracle = importlib.import_module("oracle")
    R = 1024
    o, d, n, f = ng.synthetic.sphere_rays(R, 0)
    rays = [torch.from_numpy(x).to(dev) for x in (o, d, n, f)]
    uc = np.random.default_rng(1).random((R, SC), dtype=np.float32)
    ucd = torch.from_numpy(uc).to(dev)
    p = ng.make_params(N_coarse=SC, N_fine=SF)
    bc, bf = ng.weights.glorot_blob(blob_seed[0]), ng.weights.glorot_blob(blob_seed[1])
    want, _ = oracle.nerf_forward(p, oracle.unpack_params(bc, np.float64), oracle.unpack_params(bf, np.float64),
                                  o, d, n, f, uc.astype(np.float64),
                                  np.random.default_rng(2).random((R, SF)), np.float64)
    out = {"workload": "1024 sphere rays (radius 4, direction noise N(0,0.05)), near 2, far 6, 64 stratified "
                       "samples, coarse network only (Glorot init), rgb/depth/acc maps"}
    for prec in ("fp32", "bf16", "fp8"):
        nerf = ng.NeRF(p, precision=prec, coarse_params=bc, fine_params=bf)
        for _ in range(warmup):
            nerf.render_coarse(*rays, u_coarse=ucd)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            got = nerf.render_coarse(*rays, u_coarse=ucd)
        e1.record()
        torch.cuda.synchronize()
        nerf.coarse_model.check_device_errors()
        ms = e0.elapsed_time(e1) / steps
        out[prec] = {"rays_per_s": R / (ms / 1000.0), "ms_per_pass": ms,
                     "vs_fp64_oracle": fp64_errors(got["pred_rgb"].cpu().numpy(), want["pred_rgb"])}
    return out


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""
    Q = ("index,pci.bus_id,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, bus_id=None):
        self.bus_id = (bus_id or "").lower()
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.rows = []
        if self.proc is None:
            return
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 10:
                continue
            if self.bus_id and self.bus_id[-12:] not in parts[1].lower():
                continue
            self.rows.append(parts)

    def summary(self):
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        mx = [float(r[3]) for r in self.rows if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[6 + i] == "Active"})
        loaded = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(self.rows)}


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    if args.kernel == "mlp":
        return kernel_only(args)
    if args.kernel == "train":
        return train_only(args)
    if args.kernel == "chain":
        return chain_only(args)
    import torch
    import torch.distributed as tdist

    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    if world > 1:
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    def barrier():
        if world > 1:
            tdist.barrier()

    ng = importlib.import_module("nerf-tf2_gb300")
    dev = torch.device("cuda", local_rank)
    params = ng.make_params(N_coarse=SC, N_fine=SF)
    # Scene: one sparse-density random-init network as coarse and fine.
    blob = ng.synthetic.sparse_scene_blob(SCENE_SEED, max_freq_log2=SCENE_MAX_FREQ_LOG2)
    fast = ng.NeRF(params, precision=args.path, coarse_params=blob, fine_params=blob)
    plain = ng.NeRF(params, precision="fp32", coarse_params=blob, fine_params=blob)
    # weak scaling: every rank renders its own frame (camera seed = rank)
    frame = ng.synthetic.frame_rays(rank_frame_seed(rank), H, W, FOCAL)
    R = frame[0].shape[0]
    host = [torch.from_numpy(x).pin_memory() for x in frame]
    rays = [h.to(dev) for h in host]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    n_chunks = (R + CHUNK - 1) // CHUNK

    # Learned proposal: trained (untimed) by the library's own kernels on the
    # coarse-pass weight histograms of 200k rays of this scene.
    proposal = None
    prop_info = None
    if args.proposal:
        t0 = time.perf_counter()
        tr = [torch.from_numpy(x).to(dev) for x in ng.synthetic.training_rays(100 + rank, 100, 2000)]
        g = torch.Generator(device=dev)
        g.manual_seed(0)
        uc = torch.rand(tr[0].shape[0], SC, device=dev, generator=g)
        w_t = ng.proposal.coarse_histograms(fast, *tr, uc)
        proposal = ng.ProposalNetwork(seed=7)
        losses = ng.ProposalTrainer(proposal, params, lr=3e-3).fit(*tr, uc, w_t, steps=args.proposal_steps)
        torch.cuda.synchronize()
        prop_info = {"train_rays": int(tr[0].shape[0]), "train_cameras": 100, "steps": args.proposal_steps,
                     "mode": args.proposal_mode, "gate_tau": args.gate_tau,
                     "gate_fine_draws": bool(args.gate_fine_draws),
                     "loss_first": losses[0], "loss_last": losses[-1],
                     "train_s": round(time.perf_counter() - t0, 2)}
    # kernels per chunk: plain = coarse sample (Philox draws inside), coarse
    # MLP, fine sample (coarse compositing inside), fine MLP, composite;
    # BF16/FP8 replace = proposal front end (samples, proposal density and
    # weights), fine sample, fine MLP, composite; BF16/FP8 gate = proposal
    # front end (+ coarse gate), coarse MLP, fine sample (coarse compositing
    # and fine gate inside), fine MLP, composite. The FP32 proposal paths run
    # the sampler, proposal forward and weights as three kernels.
    prop_kw = {}
    if proposal is not None:
        prop_kw = {"proposal": proposal, "proposal_mode": args.proposal_mode, "gate_tau": args.gate_tau,
                   "gate_fine_draws": bool(args.gate_fine_draws)}
    launches_per_chunk = 5 if proposal is None else (5 if args.proposal_mode == "gate" else 4) + \
        (2 if args.path == "fp32" else 0)

    def timed_steps(fn, steps, warmup):
        for i in range(warmup):
            fn(i)
        torch.cuda.synchronize()
        times = []
        for i in range(steps):
            flush.zero_()
            barrier()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn(warmup + i)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        return max_over_ranks(sum(times), world, dev) / steps

    # headline: device-resident frame through the fast path
    def step(i):
        fast.render(*rays, chunk=CHUNK, streams=args.streams, seed=1000 * i, **prop_kw)
    bus = getattr(torch.cuda.get_device_properties(dev), "pci_bus_id", None)
    with ClockSampler(str(bus) if bus is not None else None) as clk:
        ms = timed_steps(step, args.steps, args.warmup)
    value = whole_job_rate(world, R, ms)

    # end to end: pinned host rays in, maps out, through the public API
    out_host = {k: torch.empty((R, 3) if k == "rgb" else (R,), pin_memory=True) for k in ("rgb", "depth", "acc")}

    def e2e_step(i):
        dr = [h.to(dev, non_blocking=True) for h in host]
        out = fast.render(*dr, chunk=CHUNK, streams=args.streams, seed=1000 * i, **prop_kw)
        for k in out_host:
            out_host[k].copy_(out[k], non_blocking=True)
    e2e_ms = timed_steps(e2e_step, max(2, args.steps // 2), 1)
    h2d = sum(h.numel() * h.element_size() for h in host)
    d2h = sum(v.numel() * v.element_size() for v in out_host.values())

    # the plain paths: FP32 coarse+fine (the denominator) and BF16 coarse+fine
    plain_ms = timed_steps(lambda i: plain.render(*rays, chunk=CHUNK, streams=args.streams,
                                                  seed=1000 * i), args.plain_steps, 1)
    bf16_ms = timed_steps(lambda i: fast.render(*rays, chunk=CHUNK, streams=args.streams,
                                                seed=1000 * i), args.plain_steps, 1) \
        if proposal is not None else ms
    other_mode = "replace" if args.proposal_mode == "gate" else "gate"
    other_ms = timed_steps(lambda i: fast.render(*rays, chunk=CHUNK, streams=args.streams,
                                                 seed=1000 * i, proposal=proposal,
                                                 proposal_mode=other_mode, gate_tau=args.gate_tau),
                           args.plain_steps, 1) if proposal is not None else None

    # quality on every 4th image row (160k rays), same uniforms for all paths;
    # ground truth = the plain FP32 path with 512 fine samples
    rows = torch.arange(0, H, 4, device=dev)
    sub = (rows[:, None] * W + torch.arange(W, device=dev)[None, :]).reshape(-1)
    sr = [x[sub] for x in rays]
    img_plain = plain.render(*sr, chunk=CHUNK, streams=args.streams, seed=7)
    img_fast = fast.render(*sr, chunk=CHUNK, streams=args.streams, seed=7, **prop_kw)
    img_other = fast.render(*sr, chunk=CHUNK, streams=args.streams, seed=7, proposal=proposal, proposal_mode=other_mode,
                            gate_tau=args.gate_tau) if proposal is not None else None
    img_bf16 = fast.render(*sr, chunk=CHUNK, streams=args.streams, seed=7)
    gt = ng.NeRF(ng.make_params(N_coarse=SC, N_fine=512), precision="fp32", coarse_params=blob,
                 fine_params=blob).render(*sr, chunk=CHUNK, streams=args.streams, seed=9)["rgb"]
    psnr_plain, psnr_fast = ng.psnr(gt, img_plain["rgb"]), ng.psnr(gt, img_fast["rgb"])
    quality = {"rays": int(sub.numel()), "ground_truth": "plain FP32 hierarchical, 64 coarse + 512 fine",
               "psnr_plain_fp32_db": psnr_plain, "psnr_fast_db": psnr_fast,
               "psnr_gap_db": psnr_plain - psnr_fast,
               "gate_max_gap_db": 0.1, "gate_met": bool(psnr_plain - psnr_fast <= 0.1),
               "psnr_gap_bf16_plain_db": psnr_plain - ng.psnr(gt, img_bf16["rgb"]),
               "psnr_bf16_plain_db": ng.psnr(gt, img_bf16["rgb"]),
               "psnr_fast_vs_plain_db": ng.psnr(img_plain["rgb"], img_fast["rgb"]),
               "depth_mae_fast_vs_plain": float((img_plain["depth"] - img_fast["depth"]).abs().mean()),
               "mean_acc": float(img_plain["acc"].mean())}
    if proposal is not None and args.path == "bf16":
        # the same gated path with FP8-e4m3 MLP GEMMs (per-channel scales), for reference
        fp8 = ng.NeRF(params, precision="fp8", coarse_params=blob, fine_params=blob)
        fp8_ms = timed_steps(lambda i: fp8.render(*rays, chunk=CHUNK, streams=args.streams,
                                                  seed=1000 * i, **prop_kw), args.plain_steps, 1)
        img_fp8 = fp8.render(*sr, chunk=CHUNK, streams=args.streams, seed=7, **prop_kw)
        fp8.coarse_model.check_device_errors()
        quality["fp8_" + args.proposal_mode] = {
            "rays_per_s": whole_job_rate(world, R, fp8_ms), "psnr_db": ng.psnr(gt, img_fp8["rgb"]),
            "psnr_gap_db": psnr_plain - ng.psnr(gt, img_fp8["rgb"]),
            "gate_met": bool(psnr_plain - ng.psnr(gt, img_fp8["rgb"]) <= 0.1)}
    if proposal is not None and args.proposal_mode == "gate" and args.gate_fine_draws:
        # the gate as it was before the fine draws were gated: coarse samples
        # only, threshold 1e-5
        co_kw = {"proposal": proposal, "proposal_mode": "gate", "gate_tau": 1e-5, "gate_fine_draws": False}
        co_ms = timed_steps(lambda i: fast.render(*rays, chunk=CHUNK, streams=args.streams,
                                                  seed=1000 * i, **co_kw), args.plain_steps, 1)
        co_psnr = ng.psnr(gt, fast.render(*sr, chunk=CHUNK, streams=args.streams, seed=7, **co_kw)["rgb"])
        quality["gate_coarse_only_tau_1e-5"] = {"rays_per_s": whole_job_rate(world, R, co_ms), "psnr_db": co_psnr,
                                                "psnr_gap_db": psnr_plain - co_psnr,
                                                "gate_met": bool(psnr_plain - co_psnr <= 0.1)}
    # the same gated path on a literal random-init scene: separate Glorot-uniform
    # coarse and fine networks with zero biases, no density shaping, and a
    # proposal trained on that scene's coarse histograms the same way. The
    # plain FP32 path evaluates every sample whatever the scene, so its rate
    # above is this scene's denominator too.
    glorot = None
    if proposal is not None and args.glorot_scene:
        t0 = time.perf_counter()
        bc, bfn = ng.weights.glorot_blob(31), ng.weights.glorot_blob(32)
        g_fast = ng.NeRF(params, precision=args.path, coarse_params=bc, fine_params=bfn)
        g_plain = ng.NeRF(params, precision="fp32", coarse_params=bc, fine_params=bfn)
        g_prop = ng.ProposalNetwork(seed=7)
        g_loss = ng.ProposalTrainer(g_prop, params, lr=3e-3).fit(*tr, uc, ng.proposal.coarse_histograms(g_fast, *tr, uc),
                                                                  steps=args.proposal_steps)
        g_kw = {"proposal": g_prop, "proposal_mode": "gate", "gate_tau": args.gate_tau,
                "gate_fine_draws": bool(args.gate_fine_draws)}
        g_ms = timed_steps(lambda i: g_fast.render(*rays, chunk=CHUNK, streams=args.streams,
                                                   seed=1000 * i, **g_kw), args.plain_steps, 1)
        g_gt = ng.NeRF(ng.make_params(N_coarse=SC, N_fine=512), precision="fp32", coarse_params=bc,
                       fine_params=bfn).render(*sr, chunk=CHUNK, streams=args.streams, seed=9)["rgb"]
        g_img_plain = g_plain.render(*sr, chunk=CHUNK, streams=args.streams, seed=7)
        g_img = g_fast.render(*sr, chunk=CHUNK, streams=args.streams, seed=7, **g_kw)
        g_bf16 = ng.psnr(g_gt, g_fast.render(*sr, chunk=CHUNK, streams=args.streams, seed=7)["rgb"])
        g_fast.coarse_model.check_device_errors()
        gp, gf = ng.psnr(g_gt, g_img_plain["rgb"]), ng.psnr(g_gt, g_img["rgb"])
        glorot = {"scene": "coarse = Glorot-uniform blob seed 31, fine = seed 32, zero biases",
                  "path": f"{args.path}+proposal (gate, tau {args.gate_tau:g}"
                          + (", fine draws gated)" if args.gate_fine_draws else ")"), "rays_per_s": whole_job_rate(world, R, g_ms),
                  "speedup_vs_plain_fp32": plain_ms / g_ms, "psnr_plain_fp32_db": gp, "psnr_fast_db": gf,
                  "psnr_gap_db": gp - gf, "gate_met": bool(gp - gf <= 0.1),
                  f"psnr_{args.path}_plain_db": g_bf16, f"psnr_gap_{args.path}_plain_db": gp - g_bf16,
                  "depth_mae_fast_vs_plain": float((g_img_plain["depth"] - g_img["depth"]).abs().mean()),
                  "mean_acc": float(g_img_plain["acc"].mean()), "proposal_loss_last": g_loss[-1],
                  "setup_s": round(time.perf_counter() - t0, 2)}
    if proposal is not None:
        prop_info[other_mode] = {"rays_per_s": world * R / (other_ms / 1000.0),
                                 "psnr_db": ng.psnr(gt, img_other["rgb"]),
                                 "psnr_gap_db": psnr_plain - ng.psnr(gt, img_other["rgb"]),
                                 "gate_met": bool(psnr_plain - ng.psnr(gt, img_other["rgb"]) <= 0.1)}

    # errors against the FP64 oracle on 256 rays of the frame (explicit
    # uniforms): every path of this line, the gated one against the oracle's
    # gated chain (the proposal in FP64 too) and all against the plain chain
    oracle = importlib.import_module("oracle")
    sub, uc_s, uf_s = fp64_subset(rays)
    hsub = [x.cpu().numpy() for x in sub]
    p64 = oracle.unpack_params(blob, np.float64)
    _, w_plain = oracle.nerf_forward(params, p64, p64, *hsub, uc_s.astype(np.float64), uf_s.astype(np.float64),
                                     np.float64)
    ucd, ufd = torch.from_numpy(uc_s).to(dev), torch.from_numpy(uf_s).to(dev)
    fp64 = {"rays": int(sub[0].shape[0]), "uniforms": "explicit, numpy PCG64 seed 123",
            "plain_fp32": fp64_errors(plain.render(*sub, u_coarse=ucd, u_fine=ufd)["rgb"].cpu().numpy(),
                                      w_plain["pred_rgb"]),
            f"{args.path}_plain": fp64_errors(fast.render(*sub, u_coarse=ucd, u_fine=ufd)["rgb"].cpu().numpy(),
                                              w_plain["pred_rgb"])}
    if proposal is not None:
        got = fast.render(*sub, u_coarse=ucd, u_fine=ufd, **prop_kw)["rgb"].cpu().numpy()
        fp64["headline_vs_plain_chain"] = fp64_errors(got, w_plain["pred_rgb"])
        if args.proposal_mode == "gate":
            w_gate, _, _, _ = oracle.nerf_render_gated(params, proposal.params.cpu().numpy(), p64, p64, *hsub,
                                                       uc_s.astype(np.float64), uf_s.astype(np.float64),
                                                       args.gate_tau, np.float64,
                                                       gate_draws=bool(args.gate_fine_draws))
            fp64["headline_vs_gated_chain"] = fp64_errors(got, w_gate["pred_rgb"])
    cfg1 = config1(ng, dev)

    # roofline of the dominant kernel (the MLP) at the fine-pass launch shape
    nrows = CHUNK * (SC + SF)
    xyz = (torch.rand(nrows, 3, device=dev) * 4 - 2)
    dirs = torch.nn.functional.normalize(torch.randn(CHUNK, 3, device=dev), dim=1)
    mlp = fast.fine_model
    for _ in range(3):
        mlp((xyz, dirs), rows_per_dir=SC + SF)
    kt = []
    for _ in range(5):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        mlp((xyz, dirs), rows_per_dir=SC + SF)
        e1.record()
        torch.cuda.synchronize()
        kt.append(e0.elapsed_time(e1))
    mlp.check_device_errors()
    k_ms = statistics.median(kt)
    peaks = {}
    pk_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk_path):
        peaks = json.load(open(pk_path))
    achieved = nrows * FLOP_PER_SAMPLE / (k_ms / 1000.0) / 1e12
    if args.path == "bf16":
        peak, src = peaks.get("bf16_tflops"), "of measured: bf16 burst (MEASURED_PEAKS.json)"
        if peak is None:
            peak, src = 1900.0, "of fallback: 1.9 PFLOP/s bf16"
        bound = "tensor"
    else:
        clk_max = peaks.get("sm_max_mhz", 2070.0)
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        peak = sms * 128 * 2 * clk_max * 1e6 / 1e12
        src = f"FP32 FMA issue peak: {sms} SMs x 128 FMA/clk x {clk_max:.0f} MHz"
        bound = "fp32-simt"
    # DRAM bytes of one such launch are not measured in this run (that needs
    # ncu): they come from the committed capture named in traffic_source
    traffic, traffic_src = None, None
    tr_path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tr_path):
        tr = json.load(open(tr_path))
        traffic = tr.get(f"mlp_{args.path}_fine_chunk_bytes")
        if traffic is not None:
            traffic_src = "not measured in this run: " + tr.get("note", "profiles/traffic.json")

    # precision sweep: 65,536 rays x (64 coarse + 192 fine) samples, every MLP
    # precision, compensated log-sum transmittance; error against the FP32
    # path on the same uniforms, and against the FP64 oracle on 256 of the
    # rays with explicit uniforms
    sweep = None
    if args.sweep:
        p5 = ng.make_params(N_coarse=SC, N_fine=192)
        five = [x[:65536] for x in rays]
        o5, d5, n5, f5 = five
        sub5, uc5, uf5 = fp64_subset(five, n_fine=192, seed=321)
        _, w5 = oracle.nerf_forward(p5, p64, p64, *[x.cpu().numpy() for x in sub5], uc5.astype(np.float64),
                                    uf5.astype(np.float64), np.float64)
        uc5d, uf5d = torch.from_numpy(uc5).to(dev), torch.from_numpy(uf5).to(dev)
        out5, rate5, err5 = {}, {}, {}
        for prec in ("fp32", "bf16", "fp8"):
            m5 = ng.NeRF(p5, precision=prec, coarse_params=blob, fine_params=blob)
            sms = timed_steps(lambda i: m5.render(o5, d5, n5, f5, chunk=16384, seed=50 + i), 2 if prec != "fp32" else 1, 1)
            rate5[prec] = 65536 / (sms / 1000.0)
            out5[prec] = m5.render(o5, d5, n5, f5, chunk=16384, seed=77)["rgb"]
            err5[prec] = fp64_errors(m5.render(*sub5, u_coarse=uc5d, u_fine=uf5d)["rgb"].cpu().numpy(),
                                     w5["pred_rgb"])
        sweep = {"workload": "65536 rays x (64 coarse + 192 fine) samples, one frame's first 65536 rays",
                 **{prec: {"rays_per_s": rate5[prec],
                           "max_abs_rgb_vs_fp32": float((out5[prec] - out5["fp32"]).abs().max()),
                           "psnr_vs_fp32_db": ng.psnr(out5["fp32"], out5[prec]),
                           "vs_fp64_oracle_256_rays": err5[prec]} for prec in rate5}}

    # training step (model.py:127-180): 4096 rays of the scene's renders
    train = None
    if args.train_steps > 0:
        batch = [torch.from_numpy(x[:4096]).to(dev) for x in ng.synthetic.training_rays(500 + rank, 4, 1024)]
        target = plain.render(*batch, seed=3)["rgb"]
        train = {"batch_rays": 4096, "master_weights": "fp32",
                 "backward": "autograd.RenderFunction with tiles of 4096 rays (one tile: its tape is kept from "
                             "the forward); *_recompute: tiles of train_tile rays, each tile's tape recomputed "
                             "in backward", "train_tile": args.train_tile}
        for tp, tile in (("bf16", 4096), ("bf16", args.train_tile or None), ("fp32", 4096)):
            student = ng.NeRF(params, precision=tp, seed=60)
            student.backward_streams = args.streams
            tms = timed_steps(lambda i: student.train_step((tuple(batch), (target,)), tile_rays=tile),
                              args.train_steps, 1)
            student.coarse_model.check_device_errors()
            key = tp if tile == 4096 else tp + "_recompute"
            train[key] = {"rays_per_s": 4096 / (tms / 1000.0), "ms_per_step": tms,
                          "gemms": "BF16 tcgen05 GEMMs forward and backward, FP32 accumulation"
                          if tp == "bf16" else "FP32 SIMT"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, nr = cpu_render_rate(ng, frame, args.cpu_seconds)
        cpu = {"value": rate, "unit": "rays/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"first {nr} rays of the frame in 128-ray blocks, 64+128 samples; numpy "
                         "FP32 restatement of the reference (TensorFlow 2.6 is not installable "
                         "here); OpenBLAS on all host cores"}

    if rank == 0:
        mode = args.proposal_mode
        if mode == "gate":
            mode += f", tau {args.gate_tau:g}" + (", fine draws gated" if args.gate_fine_draws else "")
        path = f"{args.path}+proposal ({mode})" if proposal is not None \
            else f"{args.path} plain hierarchical"
        line = {
            "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.path, "data": "synthetic",
            "config": {"workload": WORKLOAD + "; proposal 2x64 (L=6) trained on 200k rays from 100 cameras",
                       "rays_per_step_per_gpu": R, "path": path, "streams": args.streams,
                       "l2": "512 MB buffer written between timed steps"},
            "plain_fp32": {"value": world * R / (plain_ms / 1000.0), "unit": "rays/s",
                           "speedup": plain_ms / ms},
            "bf16_plain": {"value": world * R / (bf16_ms / 1000.0), "unit": "rays/s"},
            "quality": quality,
            "glorot_scene": glorot,
            "fp64_oracle": fp64,
            "config1_coarse_pass": cfg1,
            "proposal": prop_info,
            "train_step": train,
            "precision_sweep": sweep,
            "roofline": {"kernel": f"mlp_{args.path} fine-pass launch ({nrows} rows)", "bound": bound,
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if peak else None, "peak_source": src,
                         "traffic": traffic, "traffic_source": traffic_src, "launch_ms": k_ms},
            "cpu_baseline": cpu,
            "e2e": {"value": world * R / (e2e_ms / 1000.0), "unit": "rays/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": args.steps * n_chunks * launches_per_chunk,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
