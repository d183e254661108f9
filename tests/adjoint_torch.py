"""torch.autograd.Function around the library's adjoint, for the tests only:
the differentiable compression run J(x0, v0, E, nu, log_eps, log_sigma) of a
scene, whose backward calls femmd_adjoint_backward through the C ABI."""
import numpy as np
import torch

import femmd_old_gb300 as F


def build(scene, E, nu, log_eps, log_sigma):
    """Replay 'scene' with per-disk E, nu and eps, sigma scaled by exp()."""
    es, ss = float(np.exp(log_eps)), float(np.exp(log_sigma))
    s = F.System(0)
    for name, args in scene.calls:
        if name == "set_pair_potential":
            args = ([es * e for e in args[0]],) + tuple(args[1:])
        elif name == "add_elastomer":
            args = tuple(args[:6]) + (args[6] * ss,) + tuple(args[7:])
        elif name == "set_elastomer_material":
            e = args[0]
            args = (e, float(E[e]), float(nu[e]))
        getattr(s, name)(*args)
    return s


class CompressionRun(torch.autograd.Function):
    """J = wall stress + FEA energy after 'steps' steps (checkpoint every
    'every'), plus <cx, x_N> for an optional weight field cx."""

    @staticmethod
    def forward(ctx, x0, v0, E, nu, log_eps, log_sigma, scene, steps, every, cx):
        s = build(scene, E.detach().numpy(), nu.detach().numpy(), float(log_eps), float(log_sigma))
        s.set_positions_array(x0.detach().numpy())
        s.set_velocities_array(v0.detach().numpy())
        s.adjoint_forward(steps, every)
        ws, fe = s.adjoint_observable()
        J = ws + fe
        if cx is not None:
            J += float((cx.numpy().astype(np.float64) * s.positions().astype(np.float64)).sum())
        ctx.sys = s
        ctx.cx = cx
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        g = float(gJ)
        seed = None if ctx.cx is None else (g * ctx.cx.numpy()).astype(np.float32)
        r = ctx.sys.adjoint_backward(c_wall=g, c_fea=g, xbar_final=seed)
        t = lambda a: torch.from_numpy(np.asarray(a, np.float64))  # noqa: E731
        return (t(r["x0"]), t(r["v0"]), t(r["E"]), t(r["nu"]), torch.tensor(r["log_eps"], dtype=torch.float64),
                torch.tensor(r["log_sigma"], dtype=torch.float64), None, None, None, None)
