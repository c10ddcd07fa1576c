"""tbempy: GPU (sm_103a) BEM operator apply with the reference's Python names.

Submodules: ``ThreeD`` (operators over lib/libtbem_gpu.so), ``TwoD`` (the
2D kernels on the same operators), ``meshes``
(seeded synthetic meshes), ``autograd`` (torch.autograd wrapper), ``solve``
(GMRES with FP64 iterative refinement).
"""
from . import ThreeD, TwoD, meshes  # noqa: F401
