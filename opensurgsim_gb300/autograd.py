"""Differentiation form: a multi-step implicit-Euler rollout as a ``torch.autograd.Function``.

Forward: set per-element Young's moduli E = exp(log_young) (``gbfem_set_materials_device``), start
from (x0, v0) and take ``nsteps`` steps of ``dt`` with the body's own step (FP64 or mixed form),
keeping the state every ``checkpoint_every`` steps. Backward: for each checkpoint segment, last
first, re-run the segment's steps to recover its states (with ``checkpoint_every=1`` every state is
kept, 2n doubles a step, and no step runs again), then walk them back with
``gbfem_adjoint_step`` (the transposed solve and the per-element derivative kernels), which
accumulates dL/d(log E) and dL/d(nu) and carries (dL/dx, dL/dv) to the segment's start. Gradients
flow to ``log_young``, ``x0``, ``v0`` and, when given, the per-element Poisson ratios ``poisson``
(Fem3DElementTetrahedron.cpp:204-205: nu enters K0 through lambda and mu).

On bodies whose solve is the persistent launch (the mixed form, or a batch) with corotational
elements and one Newton iteration, the forward and the backward each run as one CUDA graph inside the
library (gbfem_rollout_forward / gbfem_rollout_backward: checkpoints, segment re-runs and step
adjoints with no host round trip); other bodies take the per-step loop above.

The reference has no adjoint; the forward steps are the reference's Fem3DRepresentation::update
semantics (one Newton iteration). All tensors are float64 on the body's device.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import GbfemError


class _CudaArray:
    """A device buffer of the library exposed to torch without a copy (__cuda_array_interface__)."""

    def __init__(self, ptr: int, n: int):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 3,
                                         "strides": None}


def state_views(body):
    """(x, v) of the body as float64 torch tensors aliasing the library's device buffers."""
    xp, vp = body.device_state()
    return (torch.as_tensor(_CudaArray(xp, body.n), device=f"cuda:{body.params.device}"),
            torch.as_tensor(_CudaArray(vp, body.n), device=f"cuda:{body.params.device}"))


def _check(body, st, allow=(_lib.GBFEM_OK,)):
    if st not in allow:
        raise GbfemError(st, _lib.last_error(body.handle))


def set_young(body, log_young: torch.Tensor, poisson: torch.Tensor = None):
    """Per-element E = exp(log_young) and, if given, nu = poisson (else each element keeps its nu)."""
    young = torch.exp(log_young.detach().to(torch.float64)).contiguous()
    nu = None if poisson is None else poisson.detach().to(torch.float64).contiguous()
    torch.cuda.synchronize(young.device)
    _check(body, _lib.load().gbfem_set_materials_device(body.handle, ctypes.c_void_p(young.data_ptr()),
                                                        None if nu is None else ctypes.c_void_p(nu.data_ptr())))


def rollout_states(body, x0, v0, dt, nsteps, keep=None):
    """Step from (x0, v0); returns the final (x, v) and, if ``keep`` is a list, appends every
    intermediate state (including the first) to it."""
    xv, vv = state_views(body)
    torch.cuda.synchronize(xv.device)
    xv.copy_(x0)
    vv.copy_(v0)
    torch.cuda.synchronize(xv.device)
    if keep is not None:
        keep.append((xv.clone(), vv.clone()))
    for _ in range(nsteps):
        st = body.step(dt, 1)
        _check(body, st, (_lib.GBFEM_OK, _lib.GBFEM_CG_MAXITER))
        if keep is not None:
            keep.append((xv.clone(), vv.clone()))
    return xv.clone(), vv.clone()


def graph_rollouts(body) -> bool:
    """Whether the body's rollouts run as CUDA graphs in the library."""
    p = body.params
    return (p.element_type == _lib.ELEMENT_COROTATIONAL_TET and p.newton_max_iterations == 1 and
            (p.precision == _lib.PRECISION_MIXED or body.num_meshes > 1))


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class ImplicitRollout(torch.autograd.Function):
    """(x_T, v_T) = rollout(log_young, poisson, x0, v0); see the module docstring. ``poisson`` may
    be None (each element keeps its Poisson ratio and gets no gradient)."""

    @staticmethod
    def forward(ctx, log_young, poisson, x0, v0, body, dt, nsteps, checkpoint_every, flags=0):
        set_young(body, log_young, poisson)
        k = max(1, int(checkpoint_every))
        ctx.has_poisson = poisson is not None
        ctx.save_for_backward(log_young, poisson if poisson is not None else log_young)
        ctx.body, ctx.dt, ctx.nsteps, ctx.k, ctx.flags = body, dt, nsteps, k, int(flags)
        ctx.graph = graph_rollouts(body)
        if ctx.graph:
            dev = x0.device
            xs = x0.detach().to(torch.float64).contiguous()
            vs = v0.detach().to(torch.float64).contiguous()
            xT = torch.empty(body.n, dtype=torch.float64, device=dev)
            vT = torch.empty(body.n, dtype=torch.float64, device=dev)
            torch.cuda.synchronize(dev)
            st = _lib.load().gbfem_rollout_forward(body.handle, float(dt), int(nsteps), k, _ptr(xs), _ptr(vs), _ptr(xT),
                                                   _ptr(vT))
            _check(body, st, (_lib.GBFEM_OK, _lib.GBFEM_CG_MAXITER))
            # The library keeps the checkpoints of the body's last forward only: the token tells the
            # backward whether another rollout of the body ran in between (then it runs this one again).
            body._rollout_token = getattr(body, "_rollout_token", 0) + 1
            ctx.token, ctx.x0, ctx.v0 = body._rollout_token, xs, vs
            ctx.checkpoints = None
            return xT, vT
        checkpoints = []
        xv, vv = state_views(body)
        torch.cuda.synchronize(xv.device)
        xv.copy_(x0.detach())
        vv.copy_(v0.detach())
        torch.cuda.synchronize(xv.device)
        checkpoints.append((xv.clone(), vv.clone()))
        for t in range(nsteps):
            st = body.step(dt, 1)
            _check(body, st, (_lib.GBFEM_OK, _lib.GBFEM_CG_MAXITER))
            if (t + 1) % k == 0 and (t + 1 < nsteps or k == 1):
                checkpoints.append((xv.clone(), vv.clone()))
        ctx.checkpoints = checkpoints
        return xv.clone(), vv.clone()

    @staticmethod
    def backward(ctx, gx, gv):
        log_young, poisson = ctx.saved_tensors
        if not ctx.has_poisson:
            poisson = None
        body, dt, nsteps, k = ctx.body, ctx.dt, ctx.nsteps, ctx.k
        dev = log_young.device
        n = body.n
        lx = (gx if gx is not None else torch.zeros(n, dtype=torch.float64, device=dev)).to(torch.float64).contiguous().clone()
        lv = (gv if gv is not None else torch.zeros(n, dtype=torch.float64, device=dev)).to(torch.float64).contiguous().clone()
        glog = torch.zeros(body.num_tets, dtype=torch.float64, device=dev)
        gnu = torch.zeros(body.num_tets, dtype=torch.float64, device=dev) if poisson is not None else None
        L = _lib.load()
        set_young(body, log_young, poisson)
        if ctx.graph:
            # The library re-runs the checkpoint segments and applies the step adjoints in one graph.
            lx0 = torch.empty_like(lx)
            lv0 = torch.empty_like(lv)
            torch.cuda.synchronize(dev)
            if getattr(body, "_rollout_token", 0) != ctx.token:
                st = L.gbfem_rollout_forward(body.handle, float(dt), int(nsteps), k, _ptr(ctx.x0), _ptr(ctx.v0),
                                             _ptr(lx0), _ptr(lv0))
                _check(body, st, (_lib.GBFEM_OK, _lib.GBFEM_CG_MAXITER))
                body._rollout_token = getattr(body, "_rollout_token", 0) + 1
                ctx.token = body._rollout_token
            st = L.gbfem_rollout_backward(body.handle, _ptr(lx), _ptr(lv), _ptr(lx0), _ptr(lv0), _ptr(glog),
                                          None if gnu is None else _ptr(gnu))
            _check(body, st, (_lib.GBFEM_OK, _lib.GBFEM_CG_MAXITER))
            return glog, gnu, lx0, lv0, None, None, None, None, None
        if k == 1:
            # Every state was kept: no step runs again.
            for t in reversed(range(nsteps)):
                xt, vt = ctx.checkpoints[t]
                dv = (ctx.checkpoints[t + 1][1] - vt).contiguous()
                torch.cuda.synchronize(dev)
                st = L.gbfem_adjoint_step(body.handle, float(dt), *[ctypes.c_void_p(a.data_ptr()) for a in
                                                                     (xt, vt, dv, lx, lv, lx, lv, glog)],
                                          None if gnu is None else ctypes.c_void_p(gnu.data_ptr()), ctx.flags)
                _check(body, st, (_lib.GBFEM_OK, _lib.GBFEM_CG_MAXITER))
            torch.cuda.synchronize(dev)
            return glog, gnu, lx, lv, None, None, None, None, None
        starts = list(range(0, nsteps, k))
        for seg in reversed(range(len(starts))):
            t0 = starts[seg]
            t1 = min(t0 + k, nsteps)
            x0s, v0s = ctx.checkpoints[seg]
            states = []
            rollout_states(body, x0s, v0s, dt, t1 - t0, keep=states)
            torch.cuda.synchronize(dev)
            for t in reversed(range(t1 - t0)):
                xt, vt = states[t]
                dv = (states[t + 1][1] - vt).contiguous()
                torch.cuda.synchronize(dev)
                st = L.gbfem_adjoint_step(body.handle, float(dt), *[ctypes.c_void_p(a.data_ptr()) for a in
                                                                     (xt, vt, dv, lx, lv, lx, lv, glog)],
                                          None if gnu is None else ctypes.c_void_p(gnu.data_ptr()), ctx.flags)
                _check(body, st, (_lib.GBFEM_OK, _lib.GBFEM_CG_MAXITER))
        torch.cuda.synchronize(dev)
        return glog, gnu, lx, lv, None, None, None, None, None


def rollout(body, log_young, x0, v0, dt, nsteps, checkpoint_every=10, flags=0, poisson=None):
    """Differentiable rollout: returns (x_T, v_T) with gradients to log_young, x0, v0 and (when
    given, float64 per element) poisson. ``flags`` (e.g. STEP_TIME_PHASES) go to every adjoint step."""
    return ImplicitRollout.apply(log_young, poisson, x0, v0, body, dt, nsteps, checkpoint_every, flags)
