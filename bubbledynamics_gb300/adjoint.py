"""Phased-array gradients of the Westervelt focal loss as a torch autograd op.

The reference has no adjoint: its forward model is the Westervelt step
(W:139-236) driven by the source plane (W:62-85).  This module wraps
bd_westervelt_adjoint, the discrete adjoint of that step with sqrt(N) forward
checkpoints and per-segment recomputation, as a ``torch.autograd.Function``
whose inputs are the element phases and amplitudes of a BD_SRC_ARRAY source:

    loss = AdjointWestervelt.apply(phases, amps, problem, loss_spec, context)
    loss.backward()          # phases.grad, amps.grad

loss = sum_x w(x) E(x) with E(x) = sum over the loss window of p(x)^2 dt,
w = -1 inside the focal ball and `side_weight` on the focal plane outside
`side_radius` (so minimising it raises the focal intensity and lowers the
side lobes).  The gradient is computed by the same device call as the loss
when either input requires a gradient; otherwise only the forward runs.
"""
import numpy as np

from . import abi
from .api import Context
from .presets import WesterveltProblem


def loss_weights(shape, loss):
    """w(x) of the focal loss on a (nz, ny, nx) grid."""
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    r2 = (x - loss.focus_ix) ** 2 + (y - loss.focus_iy) ** 2 + (z - loss.focus_iz) ** 2
    w = np.zeros(shape, np.float64)
    w[(z == loss.focus_iz) & (r2 >= loss.side_radius ** 2)] = loss.side_weight
    w[r2 <= loss.focal_radius ** 2] = -1.0
    return w


def with_elements(problem: WesterveltProblem, phases, amps):
    """A copy of `problem` whose array elements have the given phases / amplitudes."""
    q = problem.copy()
    q.set_elements(problem.array("element_of_cell"), np.asarray(phases, np.float64),
                   np.asarray(amps, np.float64))
    return q


def forward_loss(context: Context, problem: WesterveltProblem, loss):
    """The focal loss from a plain forward solve (no adjoint)."""
    q = problem.copy()
    q.params.energy_mode = abi.BD_ENERGY_P2
    q.params.energy_start, q.params.energy_end = loss.window_start, loss.window_end
    q.params.peak_start = q.params.peak_end = 0
    E = context.westervelt(q, want=("energy",))["energy"].astype(np.float64)
    return float(np.sum(loss_weights(q.shape, loss) * E))


try:
    import torch

    class AdjointWestervelt(torch.autograd.Function):
        """(phases, amps) -> focal loss, with the adjoint gradient."""

        @staticmethod
        def forward(fctx, phases, amps, problem, loss, context=None):
            context = context or Context(0)
            ph = phases.detach().to("cpu", torch.float64).numpy()
            am = amps.detach().to("cpu", torch.float64).numpy()
            q = with_elements(problem, ph, am)
            need = fctx.needs_input_grad[0] or fctx.needs_input_grad[1]
            if need:
                L, gp, ga, tm = context.westervelt_adjoint(q, loss)
                fctx.save_for_backward(torch.from_numpy(gp).to(phases.device),
                                       torch.from_numpy(ga).to(amps.device))
                fctx.timings = tm
            else:
                L = forward_loss(context, q, loss)
            return torch.tensor(L, dtype=torch.float64, device=phases.device)

        @staticmethod
        def backward(fctx, grad_out):
            gp, ga = fctx.saved_tensors
            return grad_out * gp, grad_out * ga, None, None, None

except ImportError:   # torch is optional for the C ABI itself
    AdjointWestervelt = None
