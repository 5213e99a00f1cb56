"""CPU oracle for the gpurir_gb300 ISM engine.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py``.  The product package never imports it.

Parity status: pinned.  The host helpers and the trajectory overlap-add are
pinned by golden vectors made from the reference's own Python package
(tests/golden/make_golden.py).  The ISM arithmetic in ``ism_oracle.c`` is
pinned against the reference's own CUDA kernels: ``ref_kernels.py`` compiles
src/gpuRIR_cuda.cu from the reference sources into oracle/_ref and replays its
host driver on a GB300; tests/golden/reference_kernels.npz holds their outputs
(tests/golden/make_reference_kernels.py).  Fed the reference's amplitudes and
delays, the oracle's windowed sum, lookup-table fetch, envelope and tail
transform agree with those kernels to float32 rounding
(tests/test_reference_kernels.py).  cuRAND's stream is not reproduced: the
tail's noise is this engine's Philox stream, checked bit-exactly against its
host replay here and statistically against the reference's distribution.
"""
from .oracle import *  # noqa: F401,F403
