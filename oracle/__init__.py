"""CPU FP64 oracle for the qmprs MPS-encoding path.

This package is TEST INFRASTRUCTURE.  It restates, in numpy/scipy, the
algorithm of the reference project's encoding path

    qmprs/synthesis/mps_encoding/base.py        MPSEncoder.prepare_state
    qmprs/synthesis/mps_encoding/sequential.py  Sequential (layers + sweeps)
    qmprs/primitives/mps.py                     MPS primitive operations

together with the behaviour of the third-party routines those files call
(quimb 1.10.0 tensor-network operations, quick-core's ``Ket`` and
``_get_submps_indices``), which are not vendored in the reference.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline leg may import it, and only as a checker or as the timed CPU
proxy of the reference.  The GPU product path never imports it.

Modules
-------
conventions  gauge conventions, truncation rule, completions, polar factor
dense        the dense-state restatement (the parity checker for the GPU)
mpsops       the MPS-based restatement that follows the reference call by
             call (used to validate ``dense`` and as the CPU baseline)
states       seeded synthetic input families
"""
