"""Launch-shape autotuner of the CUDA substrate.

The reference has no counterpart (TensorFlow/XLA choose its kernels).  A
plan's tunable launch shapes (``gl_tuning`` in the C ABI) are:

* the fused forward + adjoint kernel's PSF correlations for the headline
  family (EPL + shear + Sersic lens light + Sersic source, planes in shared
  memory): packed FFMA2 or scalar FFMA;
* the least-squares basis kernel: one CTA of 512 threads per SM on
  whole-image parity planes, or two CTAs of 256 threads on row bands; and
  its correlation column block (16 or 20 outputs per lane);
* the least-squares Gram kernel: FP32 register tiles or tcgen05 3xTF32,
  timed on the basis shape chosen first.

On the first call for a plan shape (images, PSF sizes, model, basis
channels, batch size rounded up to a power of two, SM count and GPU name)
every candidate is timed with CUDA events on the caller's own inputs, the
fastest is applied to the plan and cached in a JSON file (``$GIGALENS_GB300
_TUNING`` or ``~/.cache/gigalens_gb300/tuning.json``).  Later plans of the
same shape take the cached choice without timing.  Tuning is skipped while
a CUDA graph is being captured (the cached or default shape is used) and
can be switched off with ``GIGALENS_GB300_AUTOTUNE=0``.
"""
import ctypes
import json
import os
import threading

import torch

from .. import _native as N

_lock = threading.Lock()
_cache = None
# counters for tests and reports: shapes timed, and cache hits
stats = {"timed": 0, "cached": 0}


def cache_path() -> str:
    p = os.environ.get("GIGALENS_GB300_TUNING")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "gigalens_gb300", "tuning.json")


def enabled() -> bool:
    return os.environ.get("GIGALENS_GB300_AUTOTUNE", "1") != "0"


def _load():
    global _cache
    if _cache is None:
        try:
            with open(cache_path()) as fh:
                _cache = json.load(fh)
        except (OSError, ValueError):
            _cache = {}
    return _cache


def _store(key, value):
    c = _load()
    c[key] = value
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        tmp = path + ".tmp%d" % os.getpid()
        with open(tmp, "w") as fh:
            json.dump(c, fh, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass   # an unwritable cache only costs a re-tune in the next process


def clear_memory_cache():
    """Forget the in-process copy of the cache (the file is re-read)."""
    global _cache
    with _lock:
        _cache = None


def get_tuning(plan) -> dict:
    t = N.gl_tuning()
    N.call("gl_plan_get_tuning", plan.handle, ctypes.byref(t))
    return {"lsq_ctas_per_sm": t.lsq_ctas_per_sm, "lsq_col_block": t.lsq_col_block, "fused_corr": t.fused_corr,
            "lsq_gram": t.lsq_gram}


def set_tuning(plan, lsq_ctas_per_sm=0, lsq_col_block=0, fused_corr=0, lsq_gram=0):
    t = N.gl_tuning(lsq_ctas_per_sm=int(lsq_ctas_per_sm), lsq_col_block=int(lsq_col_block),
                    fused_corr=int(fused_corr), lsq_gram=int(lsq_gram))
    N.call("gl_plan_set_tuning", plan.handle, ctypes.byref(t))


def _bucket(bs: int) -> int:
    b = 1
    while b < bs:
        b *= 2
    return b


def plan_key(plan, kind: str, bs: int) -> str:
    dev = torch.cuda.get_device_properties(plan.device)
    cfg = plan.launch_config(max(1, bs))
    parts = [kind, "pix=" + ",".join(str(n) for n in plan.num_pix), "ks=%d" % cfg["subkernel_side"],
             "d=%d" % plan.d, "fam=%d" % cfg["family"], "gp=%d" % cfg["global_planes"],
             "bs=%d" % _bucket(bs), "sm=%d" % dev.multi_processor_count, "gpu=%s" % dev.name]
    if kind == "lstsq":
        nb, D = ctypes.c_size_t(0), ctypes.c_int(0)
        N.call("gl_lstsq_workspace", plan.handle, 1, ctypes.byref(nb), ctypes.byref(D))
        parts.append("D=%d" % D.value)
    parts.append("models=" + plan.layout.signature())
    return "|".join(parts)


def _time_ms(fn, reps: int, warmup: int = 2) -> float:
    for _ in range(warmup):
        fn()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(reps + 1)]
    torch.cuda.synchronize()
    ev[0].record()
    times = []
    for i in range(reps):
        fn()
        ev[i + 1].record()
    torch.cuda.synchronize()
    for i in range(reps):
        times.append(ev[i].elapsed_time(ev[i + 1]))
    times.sort()
    return times[len(times) // 2]


def _choose(plan, key, candidates, bench, reps, count=True):
    """Time every candidate (a dict of set_tuning arguments), apply and cache the
    fastest.  ``count``: add one to ``stats["timed"]`` (one per tuned plan shape)."""
    results = []
    for cand in candidates:
        try:
            set_tuning(plan, **cand)
        except N.GigaLensCudaError:
            continue
        try:
            results.append((_time_ms(bench, reps), cand))
        except N.GigaLensCudaError:
            continue
    if not results:
        return None
    results.sort(key=lambda r: r[0])
    best_ms, best = results[0]
    set_tuning(plan, **best)
    _store(key, {"choice": best, "ms": best_ms, "timings": [[ms, c] for ms, c in results]})
    if count:
        stats["timed"] += 1
    return best


def _capturing() -> bool:
    try:
        return torch.cuda.is_current_stream_capturing()
    except Exception:
        return False


def ensure_lstsq(plan, x: torch.Tensor, img_id=None, reps: int = 3):
    """Apply the cached least-squares tuning of this plan shape, or time the
    candidates on ``x`` (one gl_lstsq per repetition) and cache the fastest."""
    if getattr(plan, "_tuned_lstsq", False) or not enabled():
        return
    bs = int(x.shape[0])
    key = plan_key(plan, "lstsq", bs)
    with _lock:
        hit = _load().get(key)
        if hit:
            set_tuning(plan, **hit["choice"])
            stats["cached"] += 1
            plan._tuned_lstsq = True
            return hit["choice"]
        if _capturing() or bs == 0:
            return None
        dev = x.device

        def bench():
            nb, D = ctypes.c_size_t(0), ctypes.c_int(0)
            N.call("gl_lstsq_workspace", plan.handle, bs, ctypes.byref(nb), ctypes.byref(D))
            st = bench.bufs.get(nb.value)
            if st is None:
                st = (torch.empty(nb.value, dtype=torch.uint8, device=dev),
                      torch.empty(bs, D.value, device=dev), torch.empty(bs, device=dev))
                bench.bufs[nb.value] = st
            work, co, lg = st
            N.call("gl_lstsq", plan.handle, N.ptr(x), N.ptr(img_id), bs, N.ptr(work), nb.value, N.ptr(co), None,
                   N.ptr(lg), None, N.stream_ptr())

        bench.bufs = {}
        cands = [dict(lsq_ctas_per_sm=c, lsq_col_block=cb) for c in (1, 2) for cb in (-1, 16, 20)]
        choice = _choose(plan, key, cands, bench, reps)
        if choice is not None:
            # the Gram kernel reads the basis stack the basis kernel wrote, whatever its
            # shape: time its two variants on the chosen basis shape
            choice = _choose(plan, key, [dict(choice, lsq_gram=g) for g in (2, 1)], bench, reps, count=False)
        plan._tuned_lstsq = True
        return choice


def ensure_fused(plan, z: torch.Tensor, img_id=None, reps: int = 5):
    """Apply the cached fused-kernel tuning of this plan shape, or time the
    correlation variants on ``z`` (gl_log_prob value + gradient) and cache
    the fastest.  Only the headline family with planes in shared memory has
    more than one variant."""
    if getattr(plan, "_tuned_fused", False) or not enabled():
        return
    bs = int(z.shape[0])
    cfg = plan.launch_config(max(1, bs))
    if cfg["family"] != 0 or cfg["global_planes"]:
        plan._tuned_fused = True
        return None
    key = plan_key(plan, "fused", bs)
    with _lock:
        hit = _load().get(key)
        if hit:
            set_tuning(plan, **hit["choice"])
            stats["cached"] += 1
            plan._tuned_fused = True
            return hit["choice"]
        if _capturing() or bs == 0:
            return None
        logp = torch.empty(bs, device=z.device)
        chi2 = torch.empty(bs, device=z.device)
        grad = torch.empty_like(z)

        def bench():
            N.call("gl_log_prob", plan.handle, N.ptr(z), N.ptr(img_id), bs, N.ptr(logp), N.ptr(chi2), N.ptr(grad),
                   None, N.stream_ptr())

        choice = _choose(plan, key, [dict(fused_corr=1), dict(fused_corr=2)], bench, reps)
        plan._tuned_fused = True
        return choice
