"""torch.autograd.Function over the hand-written adjoint (tds_adjoint_run): a thin check
harness, so that the simulation's loss can sit in a torch graph.

    loss = TissueLoss.apply(params, uv0, theta0, sim, face0, n_steps, r3d_target, w_pos, phi_target, w_phi)

params is a (R, 7) float64 tensor in the order GRAD_PARAMS (k_rep, k_adh, v0, mu, tau, align, eta);
uv0 (N, 2) and theta0 (N,) the initial state (3D positions follow from the chart map). The forward
sets parameters and state on the handle, runs the forward + reverse sweep once and keeps the
gradients; backward scales them by the incoming gradient. Each call restarts from (uv0, theta0)
but the noise counter of the handle keeps advancing, so repeated calls see fresh noise unless the
caller recreates the handle.
"""
import importlib

import numpy as np
import torch

_tg = importlib.import_module(__name__.rsplit(".", 1)[0])


class TissueLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, uv0, theta0, sim, face0, n_steps, r3d_target=None, w_pos=0.0, phi_target=None,
                w_phi=0.0):
        pr = params.detach().cpu().double().numpy().reshape(sim.R, len(_tg.GRAD_PARAMS))
        ps = []
        for r, base in enumerate(sim.params):
            q = _tg.Params(**{k: getattr(base, k) for k in ("radius", "r_max", "dt", "force_mode")})
            for j, k in enumerate(_tg.GRAD_PARAMS):
                setattr(q, k, float(pr[r, j]))
            ps.append(q)
        sim.set_params(ps)
        sim.set_state(uv0.detach().cpu().double().numpy(), theta0.detach().cpu().double().numpy(), face=face0)
        out = sim.adjoint(int(n_steps), r3d_target=r3d_target, w_pos=w_pos, phi_target=phi_target, w_phi=w_phi)
        ctx.save_for_backward(torch.from_numpy(out["d_params"]).to(params.dtype),
                              torch.from_numpy(out["d_uv0"]).to(uv0.dtype),
                              torch.from_numpy(out["d_theta0"]).to(theta0.dtype))
        return torch.tensor(out["loss"], dtype=torch.float64)

    @staticmethod
    def backward(ctx, g):
        dp, duv, dth = ctx.saved_tensors
        return g * dp, g * duv, g * dth, None, None, None, None, None, None, None
