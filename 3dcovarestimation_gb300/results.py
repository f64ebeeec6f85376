"""The result records the reference's command line writes after training (drop-in for the
dictionary of ``covar_processing``, ``workflow.py:477-518``, saved as ``recorded_data.pkl``;
the training checkpoint ``training_results.bin`` is ``CovarTrainer.results_dict``).

``recorded_data`` assembles the same keys from a trained :class:`~.covar.Covar`: the
eigenvectors and eigenvalues (``Covar.eigenvecs``), every image's latent coordinates and the
inverse of their covariance (``latentMAP`` with ``return_coords_covar``), the mean volume and
the dataset bookkeeping; with ground-truth eigenvectors, their normalised form, eigenvalues and
coordinates as well.  The analysis tools of the reference read this dictionary unchanged.
"""

import pickle
from typing import Any, Dict, Optional, Sequence

import torch

from .wiener_coords import latentMAP


def recorded_data(cov, dataset, mean_volume: Optional[torch.Tensor] = None, gt_eigenvecs: Optional[torch.Tensor] = None,
                  input_paths: Sequence[Optional[str]] = (None, None, None), indices=None,
                  data_sign_inverted: bool = False, lazy: bool = False, batch_size: int = 1024,
                  **latent_kwargs: Any) -> Dict[str, Any]:
    """The ``recorded_data`` dictionary of ``workflow.py:477-518`` for a trained ``cov``.
    ``dataset`` is what :func:`~.wiener_coords.latentMAP` takes; ``gt_eigenvecs`` (k, L^3 or
    k, L, L, L) unnormalised ground-truth eigenvectors, as the reference's ``GTData`` holds."""
    import os

    eigen_est, eigenval_est = cov.eigenvecs
    dev = eigen_est.device if eigen_est.is_cuda else torch.device("cuda", torch.cuda.current_device())
    eigen_est, eigenval_est = eigen_est.to(dev), eigenval_est.to(dev)
    coords_est, covar_inv_est = latentMAP(dataset, eigen_est, eigenval_est, batch_size=batch_size,
                                          return_coords_covar=True, **latent_kwargs)
    L = cov.resolution
    absolute = lambda p: os.path.abspath(p) if p is not None else None  # noqa: E731
    out = {
        "eigen_est": eigen_est.cpu().numpy(),
        "eigenval_est": eigenval_est.cpu().numpy(),
        "coords_est": coords_est.cpu().numpy(),
        "coords_covar_inv_est": covar_inv_est.cpu().numpy(),
        "mean_est": mean_volume.detach().cpu().numpy() if mean_volume is not None else None,
        "particles_path": absolute(input_paths[0]),
        "ctf_path": absolute(input_paths[1]),
        "poses_path": absolute(input_paths[2]),
        "ind": indices,
        "data_sign_inverted": data_sign_inverted,
        "lazy": lazy,
    }
    if gt_eigenvecs is not None:
        gt = gt_eigenvecs.to(dev).reshape(gt_eigenvecs.shape[0], -1)
        vals = torch.norm(gt, dim=1) ** 2
        vecs = (gt / torch.sqrt(vals).unsqueeze(1)).reshape((-1, L, L, L))
        c_gt, ci_gt = latentMAP(dataset, vecs, vals, batch_size=batch_size, return_coords_covar=True,
                                **latent_kwargs)
        out.update({"eigenvals_GT": vals.cpu().numpy(), "eigenvectors_GT": vecs.cpu().numpy(),
                    "coords_GT": c_gt.cpu().numpy(), "coords_covar_inv_GT": ci_gt.cpu().numpy()})
    return out


def save_recorded_data(data: Dict[str, Any], path: str) -> None:
    """Pickle the dictionary as ``recorded_data.pkl`` (``workflow.py:517-518``)."""
    with open(path, "wb") as f:
        pickle.dump(data, f)
