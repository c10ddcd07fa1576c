"""2D operators with the reference's Python names (tbempy.TwoD).

The reference binds the same names in both dimensions
(python_wrapper/kernels.cpp:7-31 exports them for dim 2 and 3); its 2D FMM is
FMMOperator<2,1,1> / <2,2,2> (cpp/fmm.cpp:651-652): a quadtree, translation
surfaces of ``order`` points on a circle (cpp/fmm.cpp:7-20) and the 2D
kernels below.  Points and normals are [n][2]; the operators are those of
tbempy.ThreeD, which take their dimension from the kernel.  The 2D
operators run in the plain FP64 form.
"""
import numpy as np

from .ThreeD import (DenseOperator, DirectOperator, FMMConfig, FMMGraph, FMMOperator,  # noqa: F401
                     IntegralOperator, IntegrationStrategy, Kernel, Mesh, OperatorI,
                     SparseOperator, boundary_operator, farfield_correction_operator,
                     galerkin_csr, galerkin_obs_points, galerkin_operator, gauss_facet,
                     interpolation_csr, interpolation_operator, dense_interior_operator,
                     dense_boundary_operator,
                     interior_limit_directions, mass_csr, mass_operator_scalar,
                     mass_operator_tensor, make_adaptive_integrator, make_sinh_integrator,
                     nearfield_operator, quadrature_points)


class _Kernel2D(Kernel):
    space_dim = 2


class LaplaceSingle(_Kernel2D):
    """log(r) / (2 pi) (cpp/laplace_kernels.h:66-79)."""
    kernel_id = 16


class LaplaceDouble(_Kernel2D):
    """n_src . (y - x) / (2 pi r^2) (cpp/laplace_kernels.h:82-95)."""
    kernel_id = 17


class LaplaceHypersingular(_Kernel2D):
    """(-(n_obs . n_src) / r^2 + 2 (n_src . d)(n_obs . d) / r^4) / (2 pi)
    (cpp/laplace_kernels.h:98-110)."""
    kernel_id = 18


class IdentityScalar(_Kernel2D):
    """Identity test kernel (cpp/identity_kernels.h)."""
    kernel_id = 23


class _Elastic2D(_Kernel2D):
    tensor_dim = 2

    def __init__(self, shear_modulus, poisson_ratio):
        self.shear_modulus = float(shear_modulus)
        self.poisson_ratio = float(poisson_ratio)

    def params(self):
        return np.array([self.shear_modulus, self.poisson_ratio], dtype=np.float64)


class ElasticDisplacement(_Elastic2D):
    """Plane-strain Kelvin displacement (cpp/elastic_kernels.h:21-57)."""
    kernel_id = 19


class ElasticTraction(_Elastic2D):
    """Plane-strain traction kernel (cpp/elastic_kernels.h:59-99)."""
    kernel_id = 20


class ElasticAdjointTraction(_Elastic2D):
    """Adjoint traction kernel (cpp/elastic_kernels.h:101-141)."""
    kernel_id = 21


class ElasticHypersingular(_Elastic2D):
    """Plane-strain hypersingular kernel (cpp/elastic_kernels.h:143-189)."""
    kernel_id = 22
