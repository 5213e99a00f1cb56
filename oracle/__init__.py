"""CPU oracle for the gpurir_gb300 ISM engine.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py``.  The product package never imports it.

Parity status: the host helpers and the trajectory overlap-add are pinned by
golden vectors made from the reference's own Python package
(tests/golden/make_golden.py).  The ISM arithmetic in ``ism_oracle.c`` is
PARITY UNPINNED against a run of the reference (its CUDA cannot run in the
build container and its sources are absent from the GPU host); it restates
src/gpuRIR_cuda.cu line by line and is checked with hand-derived known answers.
"""
from .oracle import *  # noqa: F401,F403
