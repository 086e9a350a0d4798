"""Lowering of a PhysicalModel to the C ABI's model descriptor, and an owning
wrapper around ``gl_plan``.

Parameter packing follows the reference (``tf/model.py:42-49``): the flat
vector holds the leaves of the parameter structure ``(lens, [lens light,]
source)`` in ``tf.nest`` order -- groups in order, profiles in order, each
profile's keys sorted.
"""
import ctypes
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from .. import _native as N
from .. import distributions as dist
from ..simulator import SimulatorConfig, base_transform, resolved_kernel


def _profile_kind(prof) -> str:
    kind = getattr(prof, "_name", None)
    if kind not in N.PROFILE_TYPES:
        raise TypeError("profile %r is not supported by the CUDA substrate" % (prof,))
    return kind


def profile_keys(prof) -> List[str]:
    """Parameter keys the profile reads from its dict (``params`` of the reference)."""
    kind = _profile_kind(prof)
    if kind == "SHAPELETS":
        keys = ["beta", "center_x", "center_y"]
        if not prof.use_lstsq:
            keys += list(prof._amp_names)
        return keys
    keys = list(N.CANONICAL_PARAMS[kind])
    if getattr(prof, "use_lstsq", False) and "Ie" in keys:
        keys.remove("Ie")
    return keys


class ModelLayout:
    """Flat-vector layout and C descriptor of a ``PhysicalModel``."""

    def __init__(self, phys_model):
        self.phys_model = phys_model
        self.has_lens_light = len(phys_model.lens_light) > 0
        groups = [(N.GL_GROUP_LENS, phys_model.lenses)]
        if self.has_lens_light:
            groups.append((N.GL_GROUP_LENS_LIGHT, phys_model.lens_light))
        groups.append((N.GL_GROUP_SOURCE, phys_model.source_light))
        self.groups = groups
        self.entries = []       # (group position, profile index, key) per column
        desc = N.gl_model_desc()
        n_prof = 0
        for gpos, (gid, profs) in enumerate(groups):
            for pi, prof in enumerate(profs):
                kind = _profile_kind(prof)
                keys = profile_keys(prof)
                cols = {}
                for k in sorted(keys):
                    cols[k] = len(self.entries)
                    self.entries.append((gpos, pi, k))
                if n_prof >= N.GL_MAX_PROFILES:
                    raise ValueError("too many profiles (max %d)" % N.GL_MAX_PROFILES)
                pd = desc.prof[n_prof]
                pd.type = N.PROFILE_TYPES[kind]
                pd.group = gid
                pd.niter = int(getattr(prof, "niter", getattr(prof, "n_max", 0)) or 0)
                pd.use_lstsq = int(bool(getattr(prof, "use_lstsq", False)))
                pd.interpolate = int(kind == "SHAPELETS" and bool(getattr(prof, "interpolate", False)))
                for i in range(N.GL_MAX_PROFILE_PARAMS):
                    pd.col[i] = -1
                for i, name in enumerate(N.CANONICAL_PARAMS[kind]):
                    pd.col[i] = cols.get(name, -1)
                if kind == "SHAPELETS" and not prof.use_lstsq:
                    # explicit amplitudes: consecutive columns (amp00, amp01, .. sort in order)
                    amp_cols = [cols[k] for k in prof._amp_names]
                    if amp_cols != list(range(amp_cols[0], amp_cols[0] + len(amp_cols))):
                        raise ValueError("shapelet amplitude columns are not consecutive")
                    pd.col[3] = amp_cols[0]
                n_prof += 1
        desc.n_profiles = n_prof
        desc.n_params = len(self.entries)
        if desc.n_params > N.GL_MAX_PARAMS:
            raise ValueError("too many parameters (max %d)" % N.GL_MAX_PARAMS)
        self.desc = desc
        self.d = desc.n_params

    def signature(self) -> str:
        """Profile types, groups and orders, e.g. for keying tuned launch shapes."""
        d = self.desc
        return ";".join("%d.%d.%d.%d.%d" % (d.prof[i].type, d.prof[i].group, d.prof[i].niter, d.prof[i].use_lstsq,
                                           d.prof[i].interpolate) for i in range(d.n_profiles))

    def split(self, params):
        """``(lens, lens_light, source)`` lists from a reference-style structure
        (``tf/simulator.py:67-72``)."""
        if self.has_lens_light:
            return [params[0], params[1], params[2]]
        return [params[0], params[1]]

    def flatten_params(self, params, device=None) -> torch.Tensor:
        """Reference-style nested params -> ``(bs, d)`` float32 CUDA tensor."""
        groups = self.split(params)
        cols = []
        for gpos, pi, k in self.entries:
            v = groups[gpos][pi][k]
            cols.append(torch.as_tensor(v, dtype=torch.float32).reshape(-1))
        bs = max(c.numel() for c in cols)
        dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        out = torch.stack([c.to(dev).expand(bs) if c.numel() == 1 else c.to(dev) for c in cols], dim=1)
        return out.contiguous()


def image_desc(sim_config: SimulatorConfig, observed=None, background_rms=1.0, exp_time=1.0, err_map=None):
    """Fill a ``gl_image_desc``; returns (desc, keep-alive host arrays)."""
    g = N.gl_image_desc()
    g.num_pix = int(sim_config.num_pix)
    g.supersample = int(sim_config.supersample or 1)
    T = base_transform(sim_config)
    for i, v in enumerate(T.reshape(-1)):
        g.transform_pix2angle[i] = float(v)
    keep = []
    k = resolved_kernel(sim_config)
    if k is not None:
        k = np.ascontiguousarray(k, dtype=np.float32)
        keep.append(k)
        g.kernel_size = int(k.shape[0])
        g.kernel = k.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    else:
        g.kernel_size = 0
        g.kernel = None
    if observed is not None:
        o = np.ascontiguousarray(np.asarray(observed, dtype=np.float32))
        if o.shape != (g.num_pix, g.num_pix):
            raise ValueError("observed image shape %s != (%d, %d)" % (o.shape, g.num_pix, g.num_pix))
        keep.append(o)
        g.observed = o.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    else:
        g.observed = None
    g.background_rms = float(background_rms)
    g.exp_time = float(exp_time)
    if err_map is not None:
        e = np.ascontiguousarray(np.asarray(err_map, dtype=np.float32))
        if e.shape != (g.num_pix, g.num_pix):
            raise ValueError("err_map shape %s != (%d, %d)" % (e.shape, g.num_pix, g.num_pix))
        keep.append(e)
        g.err_map = e.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    else:
        g.err_map = None
    return g, keep


class Plan:
    """Owns one ``gl_plan`` (device constants of a model and its images)."""

    def __init__(self, layout: ModelLayout, images: Sequence[dict], prior=None):
        lib = N.lib()
        n = len(images)
        if n < 1 or n > N.GL_MAX_IMAGES:
            raise ValueError("1..%d images per plan" % N.GL_MAX_IMAGES)
        arr = (N.gl_image_desc * n)()
        keep = []
        self.num_pix = []
        for i, im in enumerate(images):
            g, k = image_desc(**im)
            arr[i] = g
            keep.append(k)
            self.num_pix.append(g.num_pix)
        h = ctypes.c_void_p()
        N.check("gl_plan_create", lib.gl_plan_create(ctypes.byref(layout.desc), arr, n, ctypes.byref(h)))
        self.handle = h
        self.layout = layout
        self.d = layout.d
        self.device = torch.cuda.current_device()
        self.max_pix = max(p * p for p in self.num_pix)
        if prior is not None:
            self.set_prior(prior)

    def launch_config(self, bs: int) -> dict:
        """The fused kernel's launch configuration for ``bs`` samples (``gl_autotune``)."""
        r = N.gl_tune_result()
        N.call("gl_autotune", self.handle, int(bs), ctypes.byref(r))
        return {name: getattr(r, name) for name, _ in r._fields_}

    def set_prior(self, prior):
        leaves = dist.prior_leaves(prior)
        if len(leaves) != self.d:
            raise ValueError("prior has %d leaves, model has %d parameters" % (len(leaves), self.d))
        arr = (N.gl_prior_leaf * self.d)()
        for i, leaf in enumerate(leaves):
            if not isinstance(leaf, dist.Distribution):
                raise TypeError("prior leaf %d is not a supported distribution: %r" % (i, leaf))
            code, a, b, c, d = leaf.gl_leaf()
            arr[i].dist, arr[i].a, arr[i].b, arr[i].c, arr[i].d = code, a, b, c, d
        N.check("gl_plan_set_prior", N.lib().gl_plan_set_prior(self.handle, arr, self.d))

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            try:
                N.lib().gl_plan_destroy(self.handle)
            finally:
                self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
