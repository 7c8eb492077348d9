"""CPU oracle for the tTV-NESTA path -- TEST INFRASTRUCTURE ONLY.

This package restates OpenCLIPER's algorithm on the CPU (numpy/scipy) so that
the CUDA library can be checked against it.  Only tests/, the smoke() check of
__graft_entry__.py and the cpu_baseline leg of bench.py may import it, and only
to check results or as the timed CPU baseline -- never as a product code path.

Parity status: the reference's OpenCL path cannot be built or run here (no
OpenCL headers/ICD, no clFFT/CLBlast/matio), and the reference ships no golden
vectors for this path, so the restatement itself is anchored on the
reference's source (cited file:line in every function), on the documented
definitions of clFFT and CLBlast, and on libc's drand48 (see drand48.py).
The per-operator kernels are additionally pinned by compiling the reference's
own .cl sources on the host (oracle/refkernels, built into oracle/_ref/).
"""

import os as _os
from pathlib import Path as _Path


def reference_root():
    """Root of the reference source tree, or None when it is not on this machine.

    The location comes from the REFERENCE_ROOT environment variable; without it
    the recipe looks in the build container's read-only mount.  Tests that need
    the reference's own files skip when this returns None (the GPU machine has
    no reference tree)."""
    root = _Path(_os.environ.get("REFERENCE_ROOT", "/root/reference"))
    return root if root.is_dir() else None

