"""Differentiable BDDC solve (torch.autograd) of the Q1 Poisson cube with
per-element coefficients kappa_e:  K(kappa) u = f,  K = sum_e kappa_e K_e^0.

The forward pass is the C-ABI sequence (init, upload, setup, solve, download).
The backward pass reuses the forward setup: the adjoint system K lambda = dJ/du
has the same SPD operator and homogeneous Dirichlet values, so it goes through
bddcml_change_subdomain_data_c + bddcml_setup_new_data_c + bddcml_solve_c with
the forward factors and preconditioner.  The gradient
    dJ/dkappa_e = - lambda_e^T K_e^0 u_e
is formed on the GPU by bddcml_element_gradient_dev_c, which gathers the
element vectors from u and lambda (only factors and solutions are kept).

The library holds one solver per process: between a forward pass and its
backward pass no other solve may run.
"""
from __future__ import annotations

import numpy as np
import torch

from . import problems
from . import (bddcml_change_subdomain_data, bddcml_download_local_solution, bddcml_finalize, bddcml_init,
               bddcml_setup_new_data, bddcml_setup_preconditioner, bddcml_solve, element_gradient_dev, get_profile,
               get_stats, set_precision, set_profiling, upload_problem)


class PoissonCube:
    """Operator of the differentiation example: -div(kappa grad u) = 1 on the
    unit cube, u = 0 on the boundary, Q1 elements, cubic subdomains."""

    def __init__(self, num_el_per_sub_edge: int, num_sub_per_cube_edge: int, precision: int = 1,
                 tol: float = 1e-10, maxit: int = 500, device: str = "cuda"):
        self.ne, self.ns = num_el_per_sub_edge, num_sub_per_cube_edge
        self.n = num_el_per_sub_edge * num_sub_per_cube_edge
        self.precision, self.tol, self.maxit = precision, tol, maxit
        self.device = torch.device(device)
        h = 1.0 / self.n
        self.ke0 = torch.tensor(h * problems.q1_laplace_reference_matrix(), dtype=torch.float64, device=self.device)
        self.conn = torch.from_numpy(problems.cube_connectivity(self.n)).to(self.device)
        self.nelem = self.n ** 3
        self.ndof = (self.n + 1) ** 3
        self.last_iterations = None
        # per-phase device timers of the solver during the next forward pass
        # and its backward pass (bddcml_set_profiling_c)
        self.profile = False
        # after a backward pass: the library's CUDA-event totals and statistics
        # of the forward and adjoint solves, the adjoint iterations and the
        # gradient kernel's time
        self.last_profile = None
        self.last_stats = None
        self.last_adjoint_iterations = None
        self.last_gradient_ms = None

    def solve(self, kappa: torch.Tensor) -> torch.Tensor:
        """u(kappa) as a differentiable function of kappa (float64, nelem)."""
        return _BDDCSolve.apply(kappa, self)

    # -- the pieces used by the autograd function
    def _forward(self, kappa_np: np.ndarray):
        prob = problems.poisson_on_cube(self.ne, self.ns, kappa=kappa_np)
        bddcml_init(2, [prob.nsub, 1], -1, 0, 0, 0, 0)
        set_precision(self.precision)
        if self.profile:
            set_profiling(True)
        upload_problem(prob)
        bddcml_setup_preconditioner(1, 0, 1, 1, 1, 0, 0, 0)
        it, reason, _ = bddcml_solve(0, 0, self.tol, self.maxit, 50, 0, 0)
        if reason != 0:
            raise RuntimeError(f"forward BDDC solve did not converge (reason {reason})")
        self.last_iterations = it
        return prob, self._gather(prob)

    def _adjoint(self, prob, g: np.ndarray) -> np.ndarray:
        for s in prob.subdomains:
            zero = np.zeros(s.ndofs)
            bddcml_change_subdomain_data(s.isub, s.ifix, zero, g[s.isvgvn], 1, zero)
        bddcml_setup_new_data()
        it, reason, _ = bddcml_solve(0, 0, self.tol, self.maxit, 50, 0, 0)
        if reason != 0:
            raise RuntimeError(f"adjoint BDDC solve did not converge (reason {reason})")
        self.last_adjoint_iterations = it
        lam = self._gather(prob)
        self.last_profile = get_profile()
        self.last_stats = get_stats()
        return lam

    @staticmethod
    def _gather(prob) -> np.ndarray:
        u = np.zeros(prob.ndof)
        for s in prob.subdomains:
            u[s.isvgvn] = bddcml_download_local_solution(s.isub, s.ndofs)
        return u

    def element_gradient(self, u: torch.Tensor, lam: torch.Tensor) -> torch.Tensor:
        u = u.to(self.device, torch.float64).contiguous()
        lam = lam.to(self.device, torch.float64).contiguous()
        grad = torch.empty(self.nelem, dtype=torch.float64, device=self.device)
        torch.cuda.synchronize(self.device)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()  # the kernel runs on the default stream, torch's current one here
        element_gradient_dev(self.nelem, 8, self.conn.data_ptr(), self.ke0.data_ptr(), False, u.data_ptr(),
                             lam.data_ptr(), grad.data_ptr())
        ev[1].record()
        ev[1].synchronize()
        self.last_gradient_ms = ev[0].elapsed_time(ev[1])
        return grad


class _BDDCSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, kappa: torch.Tensor, op: PoissonCube):
        k = kappa.detach().to("cpu", torch.float64).numpy()
        prob, u = op._forward(k)
        ctx.op, ctx.prob = op, prob
        u_t = torch.from_numpy(u).to(kappa.device)
        ctx.save_for_backward(u_t)
        return u_t

    @staticmethod
    def backward(ctx, grad_u: torch.Tensor):
        (u_t,) = ctx.saved_tensors
        op = ctx.op
        try:
            lam = op._adjoint(ctx.prob, grad_u.detach().to("cpu", torch.float64).numpy())
        finally:
            bddcml_finalize()
        grad = op.element_gradient(u_t, torch.from_numpy(lam))
        return grad.to(u_t.device), None
