"""PyTorch autograd wrapper: seismograms as a differentiable function of the medium and the wavelet.

    sim = behf.torch_ops.Simulation(prob, precision="f32")       # grid, source position/kind, receivers
    seis = sim(moduli, wavelet)                                   # [nrec, nt] float64, physical units
    loss = 0.5 * ((seis - observed) ** 2).sum()
    loss.backward()                                               # moduli.grad, wavelet.grad

The forward pass is behf_run on the library's own context; the backward pass is behf_gradient with the
incoming gradient as the adjoint source (the exact discrete adjoint, checkpointed).  moduli: [9, nz, ny, nx]
float32 (CUDA or CPU) in the order of behf.MODULI; wavelet: [nt] float32.  The gradient with respect to the
moduli is zero in and next to the CPML slabs (the absorbing layers are not inverted).
"""
from __future__ import annotations

import numpy as np
import torch

from . import Solver


class _BehfForward(torch.autograd.Function):
    @staticmethod
    def forward(ctx, moduli, wavelet, sim):
        seis = sim._forward(moduli, wavelet)
        ctx.sim = sim
        ctx.mod_device = moduli.device
        ctx.w_device = wavelet.device
        return seis

    @staticmethod
    def backward(ctx, grad_seis):
        sim = ctx.sim
        gw, gm = sim._backward(grad_seis.detach().to("cpu", torch.float64).numpy())
        gmod = torch.from_numpy(gm.astype(np.float32)).to(ctx.mod_device)
        gwav = torch.from_numpy(gw.astype(np.float32)).to(ctx.w_device)
        return gmod, gwav, None


class Simulation:
    """A fixed grid/source/receiver set-up whose medium and wavelet are autograd inputs."""

    def __init__(self, prob, precision: str = "f32", kernel: str = "auto", checkpoint: int = 0):
        self.prob = prob
        self.nt = prob.nt
        self.solver = Solver(prob.nx, prob.ny, prob.nz, prob.h, prob.dt, radius=prob.radius, precision=precision,
                             cpml_width=prob.cpml_width, cpml_v0=prob.cpml_v0, cpml_r=prob.cpml_r,
                             src_amp_hint=float(np.abs(prob.wavelet).max()) if prob.wavelet.size else 1.0,
                             src_f0_hint=prob.f0)
        self.solver.set_kernel(kernel)
        self.solver.enable_gradient(checkpoint)
        self._rec = (np.asarray(prob.rec_ijk, np.int32), np.asarray(prob.rec_comp, np.int32))

    def close(self):
        self.solver.close()

    def __call__(self, moduli: torch.Tensor, wavelet: torch.Tensor) -> torch.Tensor:
        return _BehfForward.apply(moduli, wavelet, self)

    def _setup(self, moduli, wavelet):
        m = moduli.detach().to(torch.float32).contiguous()
        if m.is_cuda:
            self.solver.set_medium_device([int(m[q].data_ptr()) for q in range(9)])
            torch.cuda.synchronize(m.device)
        else:
            self.solver.set_medium(m.numpy())
        w = wavelet.detach().to("cpu", torch.float32).numpy()
        self.solver.set_source(self.prob.src_kind, self.prob.src, w)
        self.solver.set_receivers(self._rec[0], self._rec[1], self.nt)

    def _forward(self, moduli, wavelet):
        self._setup(moduli, wavelet)
        self.solver.reset()
        self.solver.run(self.nt)
        return torch.from_numpy(self.solver.seismograms())

    def _backward(self, grad_seis: np.ndarray):
        return self.solver.gradient(self.nt, grad_seis)
