"""GB300-native COV3D hot path: NUFFT projection / backprojection, covariance-SGD cost and
gradient, mean CG and Wiener coordinates, as hand-written sm_103a CUDA kernels behind the C ABI
of ``include/cov3d_gb300.h`` (``libcov3d_gb300.so``), with the reference package's Python API.

The directory name starts with a digit, so import it with
``importlib.import_module("3dcovarestimation_gb300")``.
"""

from . import _lib, dataset, fsc_utils, learned_pc, mean, results, synthetic, utils, wiener_coords
from .covar import Covar, Mean
from .mean import (MeanBackprojector, cg_solve, circulant_symbol, complex_conjugate_gradient,
                   correct_upsampling_padding, get_grid_correction, reconstruct_mean, reconstruct_mean_from_halfsets,
                   reconstruct_mean_from_halfsets_DDP, regularize_lhs, regularize_mean_from_halfsets, solve_mean)
from .covar_sgd import (CovarTrainer, FusedCovarStep, ProjectedCost, cost, cost_fourier_domain,
                        cost_maximum_liklihood, cost_maximum_liklihood_fourier_domain, raw_cost_fourier_domain,
                        raw_cost_maximum_liklihood_fourier_domain, trainCovar, update_fourier_reg)
from .dataset import ResidentDataset, ResidentLoader
from .nufft_plan import (BaseNufftPlan, NufftPlan, NufftPlanDiscretized, NufftSpec, NufftType, TorchNufftAdjoint,
                         TorchNufftForward, get_half_fourier_grid, nufft_adjoint, nufft_forward)
from .projection_funcs import (centered_fft2, centered_fft3, centered_ifft2, centered_ifft3, crop_image, crop_tensor,
                               get_mask_threshold, im_backward, make_nufft_plan, pad_tensor, preprocess_image_batch,
                               vol_forward)

LIB_PATH = _lib.LIB_PATH


def build(force=False):
    """Compile the CUDA library in-tree (nvcc, sm_103a)."""
    from .build import build as _build

    return _build(force=force)
