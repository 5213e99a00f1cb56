"""Differentiable RIR simulation (torch.autograd) over the CUDA adjoint kernel.

Gradients of a loss of the early (ISM) part with respect to the wall
reflection coefficients, the source and receiver positions and the source and
receiver orientations.  The backward pass recomputes image amplitudes and
delays (nothing per image is stored by the forward pass).  The diffuse tail,
if any, is produced by the forward pass but not differentiated.

    rirs = simulate_batch_torch(rooms, fs, beta, pos_src, pos_rcv)   # packed, autograd
    loss = ((rirs - target) ** 2).sum(); loss.backward()

    model = TorchBatch(rooms, fs)            # structure prepared once for a training loop
    rirs = model(beta, pos_src, pos_rcv)

``rooms`` fixes the static structure (room_sz, nb_img, Tmax, Tdiff, patterns
and the per-room source/receiver counts); beta [n_rooms, 6], pos_src
[sum n_src, 3], pos_rcv [sum n_rcv, 3] and the optional orientations are
float32 CUDA tensors.
"""
import ctypes

import numpy as np
import torch

from . import _lib, simulator
from .batch import _room_struct, layout


class _IsmBatch(torch.autograd.Function):
    @staticmethod
    def forward(ctx, beta, pos_src, pos_rcv, orV_src, orV_rcv, batch):
        out = torch.empty(batch.total, dtype=torch.float32, device=pos_src.device)
        st = torch.cuda.current_stream(pos_src.device).cuda_stream
        ptr = lambda t: t.data_ptr() if t is not None else None
        # enqueue only: beta stays on the device, descriptors were uploaded at creation
        _lib.check(_lib.load().gpurir_adjoint_forward(
            batch.handle, beta.data_ptr(), ptr(pos_src), ptr(pos_rcv), ptr(orV_src), ptr(orV_rcv),
            out.data_ptr(), ctypes.c_void_p(st)), "gpurir_adjoint_forward")
        batch._forwards += 1
        ctx.batch, ctx.forward_no = batch, batch._forwards
        ctx.save_for_backward(beta, pos_src, pos_rcv, orV_src, orV_rcv)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        batch = ctx.batch
        beta, pos_src, pos_rcv, orV_src, orV_rcv = ctx.saved_tensors
        g = grad_out.contiguous()
        dev = pos_src.device
        gb = torch.empty((batch.n_rooms, 6), dtype=torch.float32, device=dev) if ctx.needs_input_grad[0] else None
        gs = torch.empty_like(pos_src) if ctx.needs_input_grad[1] else None
        gr = torch.empty_like(pos_rcv) if ctx.needs_input_grad[2] else None
        gos = torch.empty_like(orV_src) if orV_src is not None and ctx.needs_input_grad[3] else None
        gor = torch.empty_like(orV_rcv) if orV_rcv is not None and ctx.needs_input_grad[4] else None
        ptr = lambda t: t.data_ptr() if t is not None else None
        st = torch.cuda.current_stream(dev).cuda_stream
        # no forward call on this batch since ours: its room tables (from this beta, which
        # autograd guarantees unmodified) are still on the device
        beta_ptr = None if batch._forwards == ctx.forward_no else beta.data_ptr()
        _lib.check(_lib.load().gpurir_adjoint_backward(
            batch.handle, beta_ptr, ptr(pos_src), ptr(pos_rcv), ptr(orV_src), ptr(orV_rcv),
            g.data_ptr(), ptr(gb), ptr(gs), ptr(gr), ptr(gos), ptr(gor), ctypes.c_void_p(st)),
            "gpurir_adjoint_backward")
        return gb, gs, gr, gos, gor, None


class _L2Step(torch.autograd.Function):
    """loss = scale * sum (RIRs - target)^2 with its gradients computed in the same
    fused call (gpurir_adjoint_l2_step); backward only scales them by dL/dloss."""

    @staticmethod
    def forward(ctx, beta, pos_src, pos_rcv, orV_src, orV_rcv, target, batch, scale):
        dev = pos_src.device
        out = torch.empty(batch.total, dtype=torch.float32, device=dev)
        loss = torch.empty((), dtype=torch.float32, device=dev)
        need = ctx.needs_input_grad
        gb = torch.empty((batch.n_rooms, 6), dtype=torch.float32, device=dev) if need[0] else None
        gs = torch.empty_like(pos_src) if need[1] else None
        gr = torch.empty_like(pos_rcv) if need[2] else None
        gos = torch.empty_like(orV_src) if orV_src is not None and need[3] else None
        gor = torch.empty_like(orV_rcv) if orV_rcv is not None and need[4] else None
        ptr = lambda t: t.data_ptr() if t is not None else None
        st = torch.cuda.current_stream(dev).cuda_stream
        _lib.check(_lib.load().gpurir_adjoint_l2_step(
            batch.handle, beta.data_ptr(), ptr(pos_src), ptr(pos_rcv), ptr(orV_src), ptr(orV_rcv),
            target.data_ptr(), float(scale), out.data_ptr(), loss.data_ptr(), ptr(gb), ptr(gs), ptr(gr),
            ptr(gos), ptr(gor), ctypes.c_void_p(st)), "gpurir_adjoint_l2_step")
        batch._forwards += 1
        batch.last_rirs = out
        ctx.grads = (gb, gs, gr, gos, gor)
        return loss

    @staticmethod
    def backward(ctx, grad_loss):
        return tuple(None if g is None else g * grad_loss for g in ctx.grads) + (None, None, None)


class TorchBatch:
    """The static structure of a batch (room sizes, image counts, lengths, patterns,
    per-room source/receiver counts) prepared once on the device (gpurir_adjoint);
    calling it with beta [n_rooms, 6], positions and orientations (float32 CUDA
    tensors) returns the packed RIRs with autograd through the early part.  A call
    only enqueues kernels: nothing goes through host memory and nothing waits, so a
    training step can run back to back or be recorded in a CUDA graph
    (torch.cuda.graph)."""

    def __init__(self, rooms, fs, c=343.0, sim=None):
        rooms = [dict(r, beta=r.get("beta", np.zeros(6, np.float32))) for r in rooms]
        self.n_rooms = len(rooms)
        self.offsets = layout(rooms, fs)
        self.total = int(self.offsets[-1])
        self.fs, self.c = fs, c
        self._forwards = 0   # forward calls so far (the backward reuses the latest one's room tables)
        self.sim = sim or simulator()
        self._L = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self._L.gpurir_adjoint_create(self.sim.handle, self.n_rooms, _room_struct(rooms),
                                                 float(fs), float(c), ctypes.byref(h)), "gpurir_adjoint_create")
        self.handle = h

    def __del__(self):
        L, h = getattr(self, "_L", None), getattr(self, "handle", None)
        if L is not None and h:
            L.gpurir_adjoint_destroy(h)
            self.handle = None

    def status(self):
        """Error word of the kernels (0: none); waits for them."""
        v = ctypes.c_int()
        _lib.check(self._L.gpurir_adjoint_status(self.handle, ctypes.byref(v)), "gpurir_adjoint_status")
        return v.value

    def __call__(self, beta, pos_src, pos_rcv, orV_src=None, orV_rcv=None):
        for t in (beta, pos_src, pos_rcv, orV_src, orV_rcv):
            if t is not None and (t.dtype != torch.float32 or not t.is_cuda):
                raise ValueError("beta, positions and orientations must be float32 CUDA tensors")
        contig = lambda t: t.contiguous() if t is not None else None
        return _IsmBatch.apply(beta.reshape(self.n_rooms, 6).contiguous(), contig(pos_src), contig(pos_rcv),
                               contig(orV_src), contig(orV_rcv), self)


    def l2_loss(self, beta, pos_src, pos_rcv, orV_src=None, orV_rcv=None, target=None, reduction="sum"):
        """The L2 loss of the packed RIRs against `target` (float32 CUDA tensor of the
        packed size), reduction "sum" or "mean", as a scalar tensor with autograd.
        Forward, loss, its gradient and the adjoint run in one fused call
        (gpurir_adjoint_l2_step); loss.backward() only scales the gradients it
        computed.  The RIRs of the call are left in ``self.last_rirs``."""
        for t in (beta, pos_src, pos_rcv, orV_src, orV_rcv, target):
            if t is not None and (t.dtype != torch.float32 or not t.is_cuda):
                raise ValueError("beta, positions, orientations and target must be float32 CUDA tensors")
        if target is None or target.numel() != self.total:
            raise ValueError("target must hold the batch's packed RIRs (%d values)" % self.total)
        scale = 1.0 if reduction == "sum" else 1.0 / self.total
        contig = lambda t: t.contiguous() if t is not None else None
        return _L2Step.apply(beta.reshape(self.n_rooms, 6).contiguous(), contig(pos_src), contig(pos_rcv),
                             contig(orV_src), contig(orV_rcv), target.reshape(-1).contiguous(), self, scale)

    def l2_step(self, beta, pos_src, pos_rcv, orV_src=None, orV_rcv=None, target=None, reduction="sum"):
        """One fused training step without the autograd graph: forward, the L2 loss
        against `target`, its gradient and the adjoint in one C call
        (gpurir_adjoint_l2_step).  The gradient of every input that requires grad
        is written into its ``.grad`` (allocated on the first call, overwritten on
        later ones: no zero_grad needed); returns the loss as a 0-d tensor.  The
        RIRs of the step are left in ``self.last_rirs``.  Nothing waits for the GPU:
        the host only enqueues kernels, so an optimizer step can follow at once."""
        if target is None or target.numel() != self.total:
            raise ValueError("target must hold the batch's packed RIRs (%d values)" % self.total)
        for t in (beta, pos_src, pos_rcv, orV_src, orV_rcv, target):
            if t is not None and (t.dtype != torch.float32 or not t.is_cuda or not t.is_contiguous()):
                raise ValueError("beta, positions, orientations and target must be contiguous float32 CUDA "
                                 "tensors")
        dev = pos_src.device
        if getattr(self, "_l2_bufs", None) is None or self._l2_bufs[0].device != dev:
            self._l2_bufs = (torch.empty(self.total, dtype=torch.float32, device=dev),
                             torch.empty((), dtype=torch.float32, device=dev))
        out, loss = self._l2_bufs

        def grad_of(t):
            if t is None or not t.requires_grad:
                return None
            if t.grad is None or t.grad.shape != t.shape:
                t.grad = torch.empty_like(t)
            return t.grad.data_ptr()

        ptr = lambda t: t.data_ptr() if t is not None else None
        scale = 1.0 if reduction == "sum" else 1.0 / self.total
        _lib.check(self._L.gpurir_adjoint_l2_step(
            self.handle, beta.data_ptr(), ptr(pos_src), ptr(pos_rcv), ptr(orV_src), ptr(orV_rcv),
            target.data_ptr(), scale, out.data_ptr(), loss.data_ptr(), grad_of(beta), grad_of(pos_src),
            grad_of(pos_rcv), grad_of(orV_src), grad_of(orV_rcv),
            ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)), "gpurir_adjoint_l2_step")
        self._forwards += 1
        self.last_rirs = out
        return loss


def simulate_batch_torch(rooms, fs, beta, pos_src, pos_rcv, orV_src=None, orV_rcv=None, c=343.0,
                         sim=None):
    """Packed RIRs of a batch (float32 CUDA tensor) with autograd through the early part
    (prepares the batch structure on every call; TorchBatch keeps it)."""
    return TorchBatch(rooms, fs, c, sim)(beta, pos_src, pos_rcv, orV_src, orV_rcv)


def simulate_rir_torch(room_sz, beta, pos_src, pos_rcv, nb_img, Tmax, fs, Tdiff=None,
                       spkr_pattern="omni", mic_pattern="omni", orV_src=None, orV_rcv=None, c=343.0,
                       sim=None):
    """One room, simulateRIR's arguments as tensors; returns [M_src, M_rcv, nSamples]."""
    room = dict(room_sz=np.asarray(room_sz, dtype=np.float32), beta=np.zeros(6, np.float32),
                pos_src=np.zeros((pos_src.shape[0], 3), np.float32),
                pos_rcv=np.zeros((pos_rcv.shape[0], 3), np.float32), nb_img=list(nb_img), Tmax=Tmax,
                Tdiff=Tdiff, spkr_pattern=spkr_pattern, mic_pattern=mic_pattern)
    out = simulate_batch_torch([room], fs, beta.reshape(1, 6), pos_src, pos_rcv, orV_src, orV_rcv, c,
                               sim)
    from .workloads import n_samples
    return out.view(pos_src.shape[0], pos_rcv.shape[0], n_samples(Tmax, fs))
