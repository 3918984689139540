"""Training driver of the 1D neural functional on the GPU adjoint.

Mirrors ``qedft/train/od/train.py`` and ``qedft/train/od/trainer.py``:
``create_training_step`` (``train.py:402-466``) wraps a value-and-gradient
function of the flattened network parameters for scipy's L-BFGS-B, as the
reference's ``trainer.py:150-178`` drives it; the value and gradient come from
the hand-written SCF adjoint (``qex_gb300.od.adjoint``) with the reference's
training loss (``train.py:250-323``) in place of ``jax.value_and_grad``.  The
datasets are jax_dft's ``data/od/<molecule>/*.npy`` format, loaded as
``qedft/data_io/dataset_loader.py:11-120`` does.
"""

from __future__ import annotations

import dataclasses
import logging
import os
import pickle
import time
from pathlib import Path

import numpy as np

from . import engine as eng
from .adjoint import Ks1dAdjoint, TrajectoryLoss

log = logging.getLogger(__name__)

DEFAULT_TRAIN_CONFIG = {
    # SCF (qedft/config/train_config*.yaml and create_kohn_sham_fn, train.py:84-125)
    "num_iterations": 15,
    "alpha": 0.5,
    "alpha_decay": 0.9,
    "num_mixing_iterations": 1,
    "density_mse_converge_tolerance": -1.0,
    "enforce_reflection_symmetry": True,
    "stencil": 5,
    # loss (train.py:296-318)
    "ks_iter_to_ignore": 10,
    "discount_factor": 0.9,
    # L-BFGS-B (trainer.py:164-178)
    "maxfun": 1000,
    "factr": 1.0,
    "m": 20,
    "pgtol": 1e-14,
    "maxiter": 1000,
    "save_every_n": 10,
    "checkpoint_every": 5,
}


# ---------------------------------------------------------------------------
# Datasets (jax_dft datasets.Dataset format)
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class MoleculeSet:
    """Selected molecules of a dataset (the fields the trainer reads from jax_dft's
    ``Dataset.get_molecules`` result)."""

    locations: np.ndarray          # (B, M)
    nuclear_charges: np.ndarray    # (B, M)
    total_energy: np.ndarray       # (B,)
    density: np.ndarray            # (B, N)
    external_potential: np.ndarray  # (B, N)
    distance_x100: np.ndarray      # (B,)
    grids: np.ndarray              # (N,)
    num_electrons: int

    def molecules(self):
        return [eng.Molecule1D.from_grids(self.grids, loc, z, self.num_electrons)
                for loc, z in zip(self.locations, self.nuclear_charges)]


class Dataset:
    """A molecule family stored as ``distances``, ``distances_x100``, ``grids``,
    ``locations``, ``nuclear_charges``, ``num_electrons``, ``total_energies``,
    ``densities`` and ``external_potentials`` (``.npy`` files in one folder,
    as ``data/od/{h2,h2_h2,h4}``).  ``num_grids`` crops the grid symmetrically
    about its centre."""

    FIELDS = ("distances", "distances_x100", "grids", "locations", "nuclear_charges",
              "num_electrons", "total_energies", "densities", "external_potentials")

    def __init__(self, path=None, data=None, num_grids=None, name=None):
        if (path is None) == (data is None):
            raise ValueError("give exactly one of path and data")
        if data is None:
            data = {f: np.load(os.path.join(path, f + ".npy")) for f in self.FIELDS}
        self.name = name
        self.distances = np.asarray(data["distances"], np.float64)
        self.distances_x100 = np.asarray(data["distances_x100"]).astype(np.int64)
        self.grids = np.asarray(data["grids"], np.float64)
        self.locations = np.asarray(data["locations"], np.float64)
        self.nuclear_charges = np.asarray(data["nuclear_charges"], np.float64)
        self.num_electrons = int(np.asarray(data["num_electrons"]))
        self.total_energies = np.asarray(data["total_energies"], np.float64)
        self.densities = np.asarray(data["densities"], np.float64)
        self.external_potentials = np.asarray(data["external_potentials"], np.float64)
        if num_grids is not None:
            self._crop(int(num_grids))

    def _crop(self, num_grids):
        full = self.grids.size
        if num_grids > full:
            raise ValueError(f"num_grids ({num_grids}) exceeds the stored grid ({full})")
        cut = full - num_grids
        if cut % 2:
            raise ValueError("the grid can only be cropped by an even number of points")
        sl = slice(cut // 2, full - cut // 2)
        self.grids = self.grids[sl]
        self.densities = self.densities[:, sl]
        self.external_potentials = self.external_potentials[:, sl]

    @property
    def num_samples(self):
        return self.distances.size

    def get_molecules(self, selected_distance_x100=None) -> MoleculeSet:
        if selected_distance_x100 is None:
            mask = np.ones(self.num_samples, dtype=bool)
        else:
            wanted = set(int(d) for d in selected_distance_x100)
            mask = np.array([int(d) in wanted for d in self.distances_x100])
            if int(mask.sum()) != len(wanted):
                missing = sorted(wanted - set(int(d) for d in self.distances_x100[mask]))
                raise ValueError(f"distances x100 not in the dataset: {missing}")
        return MoleculeSet(self.locations[mask], self.nuclear_charges[mask],
                           self.total_energies[mask], self.densities[mask],
                           self.external_potentials[mask], self.distances_x100[mask],
                           self.grids, self.num_electrons)


def location_center_at_grids_center_point(locations, grids) -> bool:
    """True if every molecule's nuclei are centred on the grid's centre point
    (an odd grid has one)."""
    grids = np.asarray(grids)
    if grids.size % 2 == 0:
        return False
    centre = grids[grids.size // 2]
    return bool(np.all(np.abs(np.mean(np.atleast_2d(locations), axis=1) - centre) < 1e-8))


def load_molecular_datasets(molecule_names, datasets_params, base_path=None, num_grids=None,
                            check_grid_centering=True):
    """[(dataset, train_set)] per molecule, as ``qedft/data_io/dataset_loader.py:11-120``:
    ``datasets_params[f"dataset{k}"]`` lists the training distances (x100) of
    the k-th molecule (1-based); ``num_grids`` is an int or a per-molecule dict."""
    out = []
    for k, name in enumerate(molecule_names, 1):
        n = num_grids[name] if isinstance(num_grids, dict) else num_grids
        path = Path(base_path) / name if base_path is not None else Path(name)
        try:
            ds = Dataset(path=str(path), num_grids=n, name=name)
        except Exception as e:  # noqa: BLE001 - reported with the dataset's name
            raise RuntimeError(f"Failed to load dataset for {name} from path {path}") from e
        train = ds.get_molecules(datasets_params[f"dataset{k}"])
        if check_grid_centering and not location_center_at_grids_center_point(train.locations,
                                                                              ds.grids):
            raise ValueError(f"Training set for {name} contains examples not centered at the "
                             "center of the grids.")
        out.append((ds, train))
    return out


# ---------------------------------------------------------------------------
# Parameters: flat vector <-> window-MLP layers (jax_dft np_utils.flatten)
# ---------------------------------------------------------------------------

def flatten(params):
    """(spec, flat float64 vector) of a list of (W, b) layers."""
    spec = [(np.shape(w), np.shape(b)) for w, b in params]
    flat = np.concatenate([np.concatenate([np.ravel(w), np.ravel(b)]) for w, b in params])
    return spec, flat.astype(np.float64)


def unflatten(spec, flat):
    flat = np.asarray(flat, np.float64)
    out, i = [], 0
    for ws, bs in spec:
        nw, nb = int(np.prod(ws)), int(np.prod(bs))
        out.append((flat[i:i + nw].reshape(ws), flat[i + nw:i + nw + nb].reshape(bs)))
        i += nw + nb
    if i != flat.size:
        raise ValueError("flat parameter vector does not match the spec")
    return out


# ---------------------------------------------------------------------------
# Value and gradient, training step, L-BFGS-B
# ---------------------------------------------------------------------------

def solve_config(config) -> eng.SolveConfig:
    c = {**DEFAULT_TRAIN_CONFIG, **(config or {})}
    return eng.SolveConfig(num_iterations=int(c["num_iterations"]), alpha=float(c["alpha"]),
                           alpha_decay=float(c["alpha_decay"]),
                           num_mixing_iterations=int(c["num_mixing_iterations"]),
                           density_mse_converge_tolerance=float(c["density_mse_converge_tolerance"]),
                           convention="local", stencil=int(c["stencil"]),
                           enforce_reflection_symmetry=bool(c["enforce_reflection_symmetry"]))


def create_value_and_grad_fn(xc_energy_density_fn, spec, grids, num_electrons, config=None,
                             adjoint: Ks1dAdjoint | None = None):
    """``value_and_grad_fn(flatten_params, locations, nuclear_charges,
    initial_density, target_energy, target_density) -> (loss, grad)``: the
    reference's ``jax.value_and_grad(loss_fn)`` (``trainer.py:139-143``),
    computed by the GPU adjoint.  ``xc_energy_density_fn`` is the window-MLP
    functional (as built by ``qex_gb300.networks.build_xc_functional``)."""
    from ..xc import Partial

    c = {**DEFAULT_TRAIN_CONFIG, **(config or {})}
    cfg = solve_config(c)
    loss = TrajectoryLoss(c["discount_factor"], c["ks_iter_to_ignore"])
    adj = adjoint or Ks1dAdjoint()
    grids = np.asarray(grids, np.float64)

    def value_and_grad_fn(flatten_params, locations, nuclear_charges, initial_density,
                          target_energy, target_density):
        params = unflatten(spec, flatten_params)
        mols = [eng.Molecule1D.from_grids(grids, loc, z, num_electrons)
                for loc, z in zip(locations, nuclear_charges)]
        batch = eng.PackedBatch(mols, sort=False)
        n0 = None if initial_density is None else np.asarray(initial_density).reshape(-1)
        res = adj.value_and_grad(batch, Partial(xc_energy_density_fn, params=params), cfg,
                                 np.asarray(target_energy), np.asarray(target_density).reshape(-1),
                                 checkpoint_every=int(c["checkpoint_every"]), loss=loss,
                                 initial_density=n0)
        return res.loss, res.grad

    return value_and_grad_fn


def create_training_step(value_and_grad_fn, train_set: MoleculeSet, initial_density,
                         save_every_n: int, initial_checkpoint_index: int = 0,
                         checkpoint_dir: str | None = None, spec=None, ckpt_prefix: str = "ckpt"):
    """``np_value_and_grad_fn(flatten_params) -> (loss, grad)`` for L-BFGS-B, with
    checkpoints of the unflattened parameters every ``save_every_n`` calls
    (``qedft/train/od/train.py:402-466``)."""
    loss_record = []

    def np_value_and_grad_fn(flatten_params):
        start = time.time()
        loss, grad = value_and_grad_fn(flatten_params, locations=train_set.locations,
                                       nuclear_charges=train_set.nuclear_charges,
                                       initial_density=initial_density,
                                       target_energy=train_set.total_energy,
                                       target_density=train_set.density)
        step = initial_checkpoint_index + len(loss_record)
        log.info("step %d, loss %s in %.3f sec", step, loss, time.time() - start)
        if checkpoint_dir and len(loss_record) % save_every_n == 0:
            os.makedirs(checkpoint_dir, exist_ok=True)
            with open(f"{checkpoint_dir}/{ckpt_prefix}-{step:05d}", "wb") as fh:
                pickle.dump(unflatten(spec, flatten_params) if spec is not None
                            else np.asarray(flatten_params), fh)
        loss_record.append(loss)
        return float(loss), np.asarray(grad, dtype=np.float64)

    np_value_and_grad_fn.loss_record = loss_record
    return np_value_and_grad_fn


def initial_density(train_set: MoleculeSet, config=None, engine: eng.Ks1dEngine | None = None):
    """Non-interacting densities of the set's external potentials (jax_dft
    ``scf.get_initial_density(states, method='noninteracting')``), packed."""
    import torch

    c = {**DEFAULT_TRAIN_CONFIG, **(config or {})}
    e = engine or eng.default_engine()
    batch = eng.PackedBatch(train_set.molecules(), sort=False)
    v = torch.as_tensor(np.asarray(train_set.external_potential, np.float64).reshape(-1),
                        device=batch.device)
    n0, _, _, _ = e.noninteracting(batch, v, int(c["stencil"]))
    return n0.cpu().numpy()


def train(xc_energy_density_fn, init_params, train_set: MoleculeSet, config=None,
          checkpoint_dir=None):
    """L-BFGS-B over the flattened parameters (``qedft/train/od/trainer.py:164-178``).
    Returns (params, loss, info) as ``scipy.optimize.fmin_l_bfgs_b``."""
    import scipy.optimize

    c = {**DEFAULT_TRAIN_CONFIG, **(config or {})}
    spec, flat0 = flatten(init_params)
    vg = create_value_and_grad_fn(xc_energy_density_fn, spec, train_set.grids,
                                  train_set.num_electrons, c)
    n0 = initial_density(train_set, c)
    step = create_training_step(vg, train_set, n0, save_every_n=int(c["save_every_n"]),
                                checkpoint_dir=checkpoint_dir, spec=spec)
    x, f, info = scipy.optimize.fmin_l_bfgs_b(step, x0=flat0, maxfun=int(c["maxfun"]),
                                              factr=float(c["factr"]), m=int(c["m"]),
                                              pgtol=float(c["pgtol"]),
                                              maxiter=int(c["maxiter"]))
    info["loss_record"] = list(step.loss_record)
    return unflatten(spec, x), f, info
