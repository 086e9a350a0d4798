"""Benchmark: lik+grad evaluations per second at 4096 chains x 90x90 pixels.

Workload (the reference's headline configuration for this path): 90x90 base
pixels at 0.065"/px, supersampling 2, Gaussian PSF of FWHM 0.1" (21x21 at
base scale; the supersampled 41x41 kernel is generated directly on the fine
grid), EPL(50) + external shear, elliptical Sersic lens light and source;
4096 chains drawn from the configuration's parameter distributions;
observed image = one seeded truth draw + Poisson noise at 1000 s + Gaussian
background 0.2.  A step is one evaluation of the log posterior and its
gradient for all 4096 chains: ONE launch of the fused forward+adjoint kernel
(``gl_log_prob`` with a gradient).

  value  whole-job evals/s with inputs resident in HBM, timed with CUDA events
         on the launching stream; L2 is flushed (256 MiB write) between steps
  e2e    the same through the public API (``ForwardProbModel.log_prob`` +
         autograd backward) with pinned host buffers: H2D of z, D2H of
         logp, chi^2 and the gradient inside the timed region
  roofline  algorithmic FP32 flop per eval (forward + adjoint, the
         minimal strided PSF form) x chains / kernel time, against the FP32
         FMA peak measured live by a probe kernel at the same clocks
  cpu_baseline  the float32 PyTorch-CPU restatement (autograd) on a bounded
         sample of the same workload, all host threads

``--impl reference`` times the reference's CPU path; TensorFlow is not
installed, so that is the same float32 CPU restatement of the reference's
algorithm (``kind: port``), on all host threads.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "lik+grad evals/s @4096x90^2px"
UNIT = "evals/s"
N_PIX, SS, DELTA, FWHM, PSF_BASE = 90, 2, 0.065, 0.1, 21
BG_RMS, EXP_TIME, NITER = 0.2, 1000.0, 50


def workload_prior():
    """A prior whose supports hold the configuration's distributions (the
    bijectors of log_prob need one); chains are drawn from the configuration
    itself by ``draw_chains``."""
    from gigalens_gb300 import distributions as tfd

    ie_ll = tfd.LogNormal(0.75 * math.log(10), 0.75 * math.log(10) / math.sqrt(3))
    ie_src = tfd.LogNormal(1.25 * math.log(10), 0.75 * math.log(10) / math.sqrt(3))
    return tfd.JointDistributionSequential([
        tfd.JointDistributionSequential([
            tfd.JointDistributionNamed(dict(theta_E=tfd.Uniform(1.0, 1.6), gamma=tfd.Uniform(1.8, 2.3),
                                            e1=tfd.Normal(0, 0.1), e2=tfd.Normal(0, 0.1),
                                            center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05))),
            tfd.JointDistributionNamed(dict(gamma1=tfd.Normal(0, 0.05), gamma2=tfd.Normal(0, 0.05)))]),
        tfd.JointDistributionSequential([tfd.JointDistributionNamed(dict(
            R_sersic=tfd.Uniform(0.5, 1.5), n_sersic=tfd.Uniform(2, 6), e1=tfd.Normal(0, 0.1),
            e2=tfd.Normal(0, 0.1), center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05), Ie=ie_ll))]),
        tfd.JointDistributionSequential([tfd.JointDistributionNamed(dict(
            R_sersic=tfd.Uniform(0.05, 0.4), n_sersic=tfd.Uniform(0.5, 4),
            e1=tfd.TruncatedNormal(0, 0.15, -0.5, 0.5), e2=tfd.TruncatedNormal(0, 0.15, -0.5, 0.5),
            center_x=tfd.Uniform(-0.3, 0.3), center_y=tfd.Uniform(-0.3, 0.3), Ie=ie_src))]),
    ])


def draw_chains(n, seed):
    """Parameter structure of n chains from the configuration's distributions."""
    import torch

    r = np.random.default_rng(seed)
    f = lambda a: torch.tensor(np.asarray(a, dtype=np.float32))
    lens = {"theta_E": f(r.uniform(1.0, 1.6, n)), "gamma": f(r.uniform(1.8, 2.3, n)),
            "e1": f(r.normal(0, 0.1, n)), "e2": f(r.normal(0, 0.1, n)),
            "center_x": f(r.normal(0, 0.05, n)), "center_y": f(r.normal(0, 0.05, n))}
    sh = {"gamma1": f(r.normal(0, 0.05, n)), "gamma2": f(r.normal(0, 0.05, n))}
    ll = {"R_sersic": f(r.uniform(0.5, 1.5, n)), "n_sersic": f(r.uniform(2, 6, n)),
          "e1": f(r.normal(0, 0.1, n)), "e2": f(r.normal(0, 0.1, n)),
          "center_x": f(r.normal(0, 0.05, n)), "center_y": f(r.normal(0, 0.05, n)),
          "Ie": f(10 ** r.uniform(0, 1.5, n))}
    src = {"R_sersic": f(r.uniform(0.05, 0.4, n)), "n_sersic": f(r.uniform(0.5, 4, n)),
           "e1": f(np.clip(r.normal(0, 0.15, n), -0.49, 0.49)), "e2": f(np.clip(r.normal(0, 0.15, n), -0.49, 0.49)),
           "center_x": f(r.uniform(-0.3, 0.3, n)), "center_y": f(r.uniform(-0.3, 0.3, n)),
           "Ie": f(10 ** r.uniform(0.5, 2, n))}
    return [[lens, sh], [ll], [src]]


def gaussian_psf(fwhm, pixel, side):
    sigma = fwhm / (2.0 * math.sqrt(2.0 * math.log(2.0)))
    r = (np.arange(side) - (side - 1) / 2.0) * pixel
    g = np.exp(-0.5 * (r / sigma) ** 2)
    k = np.outer(g, g)
    return (k / k.sum()).astype(np.float32)


def epl_terms(e1, e2, cap=NITER):
    """The reference's term-count rule (tf/profiles/mass/epl.py:41), float32."""
    e1 = np.asarray(e1, np.float32)
    e2 = np.asarray(e2, np.float32)
    c = np.clip(np.sqrt(e1 * e1 + e2 * e2), np.float32(0), np.float32(1))
    q = (1 - c) / (1 + c)
    f = (1 - q) / (1 + q)
    with np.errstate(divide="ignore"):
        niter = np.float32(np.log(np.float32(1e-12))) / np.log(np.float32(f.max())) + np.float32(2)
    if not niter > 1:
        return 0
    return int(min(cap, math.ceil(float(niter)) - 1))


def flops_per_eval(K, n=N_PIX, ss=SS, k=2 * PSF_BASE - 1):
    """Algorithmic FP32 flop of one forward + adjoint evaluation:
    F_px = 84 + 10 K per supersampled pixel (lens + light), the PSF+binning
    as one strided correlation with the (k+ss-1)^2 combined kernel at the
    N^2 outputs, 12 flop per output for the likelihood; the adjoint is twice
    the pixel work (recompute + reverse) plus one transposed correlation."""
    Ps, P = (ss * n) ** 2, n * n
    Fpx = 84 + 10 * K
    Fpsf = 2 * P * (k + ss - 1) ** 2
    Flik = 12 * P
    fwd = Ps * Fpx + Fpsf + Flik
    adj = 2 * Ps * Fpx + Fpsf + Flik
    return fwd, adj


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        rows = [l.split(",") for l in open(self.f.name).read().strip().splitlines() if l.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() in ("active", "1"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_port_rate(n_chains, seconds_hint=None):
    """Float32 PyTorch-CPU restatement (oracle) of lik+grad on n chains."""
    import torch

    from oracle import lens_oracle as O
    from gigalens_gb300 import distributions as tfd

    torch.set_num_threads(os.cpu_count() or 1)
    model = dict(lenses=[("EPL", {"niter": NITER}), ("SHEAR", {})], lens_light=[("SERSIC_ELLIPSE", {})],
                 source_light=[("SERSIC_ELLIPSE", {})])
    ksub = gaussian_psf(FWHM, DELTA / SS, 2 * PSF_BASE - 1)
    cfg = O.SimConfig(DELTA, N_PIX, SS, ksub.astype(np.float32))
    xs = draw_chains(n_chains, seed=1)
    truth = draw_chains(1, seed=0)
    im = O.simulate(model, cfg, [[{k: v.double() for k, v in d.items()} for d in g] for g in truth])[0].numpy()
    obs = make_observed(im)
    x = torch.stack([v.reshape(-1) for v in tfd.flatten(xs)], dim=1).float()
    K = epl_terms(x[:, 2].numpy(), x[:, 3].numpy())

    def once():
        xx = x.clone().requires_grad_(True)
        ll, chi2 = O.forward_log_likelihood_flat(model, cfg, xx, obs.astype(np.float32), BG_RMS, EXP_TIME,
                                                 dtype=torch.float32)
        ll.sum().backward()
        return xx.grad

    once()
    t0 = time.perf_counter()
    reps = 0
    while True:
        once()
        reps += 1
        el = time.perf_counter() - t0
        if seconds_hint is None or el > seconds_hint or reps >= 50:
            break
    el = time.perf_counter() - t0
    return n_chains * reps / el, torch.get_num_threads(), reps, el, K


def make_observed(im_truth):
    rng = np.random.default_rng(1)
    counts = rng.poisson(np.clip(im_truth, 0, None) * EXP_TIME) / EXP_TIME
    return (counts + rng.normal(scale=BG_RMS, size=im_truth.shape)).astype(np.float32)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    n = args.ref_chains
    rates = []
    K = None
    for i in range(args.warmup + args.steps):
        r, cores, reps, el, K = cpu_port_rate(n, seconds_hint=args.ref_seconds)
        if i >= args.warmup:
            rates.append(r)
    val = statistics.median(rates)
    line = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 4096.0 / val * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "4096 chains x 90x90 px, ss=2, PSF 41x41 (supersampled), EPL(50)+shear, "
                                   "SersicEllipse lens light + source; CPU sample of %d chains per step" % n,
                       "epl_terms": K},
            "impl": "reference",
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d chains per step, float32 PyTorch-CPU restatement of the reference's "
                                       "TF path with autograd (TensorFlow is not installed)" % n},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import torch.distributed as tdist

    ws, rank, local = dist_env()
    if ws > 1:
        tdist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from gigalens_gb300 import _native as N
    from gigalens_gb300 import distributions as tfd
    from gigalens_gb300.model import PhysicalModel
    from gigalens_gb300.simulator import SimulatorConfig
    from gigalens_gb300.cuda.model import ForwardProbModel, log_prob_and_grad
    from gigalens_gb300.cuda.profiles.light import sersic
    from gigalens_gb300.cuda.profiles.mass import epl, shear
    from gigalens_gb300.cuda.simulator import LensSimulator

    bs = args.chains
    phys = PhysicalModel([epl.EPL(NITER), shear.Shear()], [sersic.SersicEllipse()], [sersic.SersicEllipse()])
    ksub = gaussian_psf(FWHM, DELTA / SS, 2 * PSF_BASE - 1)
    cfg = SimulatorConfig(delta_pix=DELTA, num_pix=N_PIX, supersample=SS, kernel_supersampled=ksub)
    truth_sim = LensSimulator(phys, cfg, bs=1)
    truth = draw_chains(1, seed=0)
    im = truth_sim.simulate(truth).cpu().numpy().astype(np.float64)
    obs = make_observed(im)
    prior = workload_prior()
    pm = ForwardProbModel(prior, obs, background_rms=BG_RMS, exp_time=EXP_TIME)
    sim = LensSimulator(phys, cfg, bs=bs)
    plan = sim.prob_plan(pm)
    xs = draw_chains(bs, seed=1 + rank)
    z = pm.bij.inverse(xs).to(torch.float32).to(dev).contiguous()
    K = epl_terms(xs[0][0]["e1"].numpy(), xs[0][0]["e2"].numpy())
    logp = torch.empty(bs, device=dev)
    chi2 = torch.empty(bs, device=dev)
    grad = torch.empty_like(z)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def step():
        log_prob_and_grad(plan, z, logp, chi2, grad)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    finite = bool(torch.isfinite(logp).all()) and bool(torch.isfinite(grad).all())

    # ---- device-resident timing: one fused launch per step, L2 flushed between
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    if ws > 1:
        tdist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall0 = time.perf_counter()
    for i in range(args.steps):
        flush.fill_(float(i))
        starts[i].record(stream)
        step()
        ends[i].record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    if ws > 1:
        tdist.barrier()
    clk = clocks.stop()
    times = [s.elapsed_time(e) for s, e in zip(starts, ends)]   # ms
    t_step = sum(times) / len(times)
    if ws > 1:
        tt = torch.tensor([t_step], device=dev)
        tdist.all_reduce(tt, op=tdist.ReduceOp.MAX)
        t_step = float(tt)
    value = ws * bs / (t_step * 1e-3)

    # ---- FP32 peak (probe kernel, same clocks)
    probe_out = torch.empty(4096, device=dev)
    flops = ctypes_double()
    for _ in range(2):
        N.call("gl_probe_fp32_fma", N.ptr(probe_out), 2000, 4, flops, N.stream_ptr())
    pe0, pe1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pe0.record(stream)
    N.call("gl_probe_fp32_fma", N.ptr(probe_out), 2000, 4, flops, N.stream_ptr())
    pe1.record(stream)
    torch.cuda.synchronize()
    fp32_peak = flops.value / (pe0.elapsed_time(pe1) * 1e-3) / 1e12

    # ---- e2e through the public API with pinned host buffers
    z_host = z.cpu().pin_memory()
    out_host = torch.empty((bs, 2 + z.shape[1]), dtype=torch.float32).pin_memory()
    z_dev = torch.empty_like(z)
    e2e_times = []
    for i in range(args.warmup + args.steps):
        flush.fill_(float(i))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        z_dev.copy_(z_host, non_blocking=True)
        zz = z_dev.requires_grad_(True)
        lp, c2 = pm.log_prob(sim, zz)
        (gz,) = torch.autograd.grad(lp.sum(), zz)
        dev_out = torch.cat([lp[:, None], c2[:, None], gz], dim=1)
        out_host.copy_(dev_out, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        z_dev = z_dev.detach()
        if i >= args.warmup:
            e2e_times.append(e0.elapsed_time(e1))
    t_e2e = sum(e2e_times) / len(e2e_times)
    if ws > 1:
        tt = torch.tensor([t_e2e], device=dev)
        tdist.all_reduce(tt, op=tdist.ReduceOp.MAX)
        t_e2e = float(tt)
    e2e_value = ws * bs / (t_e2e * 1e-3)

    fwd, adj = flops_per_eval(K)
    achieved = (fwd + adj) * bs / (t_step * 1e-3) / 1e12

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        r, cores, reps, el, _ = cpu_port_rate(args.cpu_chains, seconds_hint=args.cpu_seconds)
        cpu = {"value": r, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "%d chains x %d repetitions (%.1f s), float32 PyTorch-CPU restatement with autograd"
                         % (args.cpu_chains, reps, el)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "4096 chains x 90x90 px, ss=2, PSF 41x41 (supersampled Gaussian, FWHM "
                                       "0.1\"), EPL(50)+shear, SersicEllipse lens light + source; one fused "
                                       "forward+adjoint launch per step",
                           "chains_per_gpu": bs, "epl_terms": K, "l2": "flushed between steps (256 MiB write)",
                           "wall_s_timed": t_wall, "finite": finite},
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(z.numel() * 4),
                        "d2h_bytes_per_step": int(out_host.numel() * 4),
                        "api": "ForwardProbModel.log_prob + torch.autograd.grad, pinned host buffers"},
                "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                             "frac": achieved / fp32_peak, "traffic": None,
                             "flop_per_eval": fwd + adj,
                             "peak_source": "FP32 FMA probe kernel measured in this run (MEASURED_PEAKS.json "
                                            "holds no FP32 figure)"},
                "cpu_baseline": cpu,
                "gpu_launches": args.steps,
                "clocks": clk}
        print(json.dumps(line), flush=True)
    if ws > 1:
        tdist.destroy_process_group()


def ctypes_double():
    import ctypes

    return ctypes.c_double(0.0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--chains", type=int, default=4096)
    ap.add_argument("--cpu-chains", type=int, default=8)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-chains", type=int, default=8)
    ap.add_argument("--ref-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
