"""Fractional (Fermi-Dirac) orbital occupations, ``qedft/train/td/fermi.py``.

The chemical-potential search runs on the GPU (``qex_td_fermi_occupations``,
one CTA per spectrum, FP64); the three reference entry points map to its
modes.  Energies may be a 1D spectrum or a (batch, n) stack; results come
back as device tensors (occupations) and floats or (batch,) tensors.
The small elementwise helpers of the reference module are provided on
device tensors as well.
"""

from __future__ import annotations

from .. import _native as N
from . import _lib
from .numint import _dev


def _run(mo_energy, n_electrons, theta, mu, mu_shift, step, max_steps, mode):
    torch = N.require_cuda()
    e = _dev(mo_energy, torch.float64)
    single = e.dim() == 1
    if single:
        e = e[None]
    e = e.contiguous()
    B, n = e.shape
    ne = torch.as_tensor(n_electrons, dtype=torch.float64, device="cuda").reshape(-1)
    if ne.numel() == 1:
        ne = ne.expand(B).contiguous()
    mu_in = None if mu is None else torch.as_tensor(mu, dtype=torch.float64,
                                                    device="cuda").reshape(-1).expand(B).contiguous()
    occ = torch.empty_like(e)
    mu_out = torch.empty(B, dtype=torch.float64, device="cuda")
    entr = torch.empty_like(mu_out)
    loss = torch.empty_like(mu_out)
    st = torch.zeros(B, dtype=torch.int32, device="cuda")
    N.check(_lib.lib().qex_td_fermi_occupations(
        B, n, _lib.p(e), _lib.p(ne), float(theta), _lib.p(mu_in) if mu_in is not None else None,
        float(mu_shift), float(step), int(max_steps), int(mode), _lib.p(occ), _lib.p(mu_out),
        _lib.p(entr), _lib.p(loss), _lib.p(st), _lib.stream()), "qex_td_fermi_occupations")
    if single:
        return occ[0], entr[0], mu_out[0], loss[0], st[0]
    return occ, entr, mu_out, loss, st


def optimize_fermi_occupations(mo_energy, n_electrons, theta=0.04, mu_initial=None,
                               mu_shift=0.001, step_grad=0.6, max_steps=100, tol=1e-9):
    """``fermi.py:145-219``: stops once the loss is below 1e-9 (the reference's
    default ``tol``); ValueError when it ends above 1e-2."""
    if tol != 1e-9:
        raise ValueError("the GPU search stops at the reference's tolerance, 1e-9")
    occ, entr, mu, loss, st = _run(mo_energy, n_electrons, theta, mu_initial, mu_shift,
                                   step_grad, max_steps, 0)
    if bool((st != 0).any()):
        raise ValueError(f"Fermi occupation optimization failed: loss={loss.cpu().numpy()}. "
                         "Try increasing max_steps or adjusting parameters.")
    return occ, entr, mu, loss


def get_fractional_occupations(mo_energy, n_electrons, frac_mo_occ=1, frac_theta=0.04,
                               frac_mu=None, frac_mu_shift=0.001, frac_step_grad=0.6,
                               frac_max_steps=100):
    """``fermi.py:222-298``: 1 -> Fermi-Dirac search, an array -> the given
    occupations, None -> aufbau filling (a fractional remainder in the last
    orbital).  Returns (mo_occ, energy_entr, mu_opt, loss_final)."""
    torch = N.require_cuda()
    if frac_mo_occ is None:
        e = _dev(mo_energy, torch.float64)
        occ = torch.zeros_like(e)
        rem = float(n_electrons)
        full = min(int(rem // 2), e.shape[-1])
        occ[..., :full] = 2.0
        rem -= 2.0 * full
        if rem > 0.0 and full < e.shape[-1]:
            occ[..., full] = rem
        return occ, 0.0, None, None
    if isinstance(frac_mo_occ, (int, float)) and not isinstance(frac_mo_occ, bool) \
            and frac_mo_occ == 1:
        return optimize_fermi_occupations(mo_energy, n_electrons, frac_theta, frac_mu,
                                          frac_mu_shift, frac_step_grad, frac_max_steps)
    if hasattr(frac_mo_occ, "shape"):
        return _dev(frac_mo_occ, torch.float64), 0.0, None, None
    raise ValueError(f"frac_mo_occ={frac_mo_occ} not implemented. "
                     "Use None, 1 (for Fermi-Dirac), or an array.")


def get_fractional_occupations_jax(mo_energy, n_electrons, theta, frac_mu, frac_mu_shift,
                                   frac_step_grad, frac_max_steps):
    """``fermi.py:301-390``: min(frac_max_steps, 100) damped Newton steps."""
    occ, entr, mu, loss, _ = _run(mo_energy, n_electrons, theta, frac_mu, frac_mu_shift,
                                  frac_step_grad, frac_max_steps, 1)
    return occ, entr, mu, loss


def get_fractional_occupations_jax_stable(mo_energy, n_electrons, theta, frac_mu,
                                          frac_mu_shift, frac_step_grad, frac_max_steps):
    """``fermi.py:393-497``: Newton from the HOMO/LUMO midpoint with a
    theta = 0.01 fallback; the loss is reported as 0."""
    occ, entr, mu, loss, _ = _run(mo_energy, n_electrons, theta, frac_mu, frac_mu_shift,
                                  frac_step_grad, frac_max_steps, 2)
    return occ, entr, mu, loss


# elementwise helpers of the reference module (device tensors)

def fermi_function4entropy(energy, mu, theta):
    torch = N.require_cuda()
    return 1.0 / (1.0 + torch.exp((_dev(energy, torch.float64) - mu) / theta))


def fermi_function(energy, mu, theta):
    return 2.0 * fermi_function4entropy(energy, mu, theta)


def make_occ_fermi(mu, mo_energy, theta):
    return fermi_function(mo_energy, mu, theta)


def loss_fermi_function(mu, mo_energy, n, theta):
    return (n - fermi_function(mo_energy, mu, theta).sum()) ** 2


def entropy(f):
    """f ln f + (1 - f) ln(1 - f), with 0 ln 0 = 0."""
    torch = N.require_cuda()
    f = _dev(f, torch.float64)
    return torch.special.xlogy(f, f) + torch.special.xlogy(1.0 - f, 1.0 - f)


def etropic_energy_contribution(mu, mo_energy, theta):
    return theta * (2.0 * entropy(fermi_function4entropy(mo_energy, mu, theta))).sum()
