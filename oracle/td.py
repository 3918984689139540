"""NumPy float64 restatement of the 3D numint / generalized-eigh / DIIS / rdm1
SCF pieces of the reference (test oracle; the CUDA product path never imports
this module).

Each function cites the reference file:line it follows.  pyscf / pyscfad are
not installed anywhere this project runs, so the one-electron and
two-electron integrals come from the synthetic model of
``synthetic_molecule`` (same inputs for the oracle and the GPU path).
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np

SLATER_CX = 0.75 * (3.0 / math.pi) ** (1.0 / 3.0)


# ----------------------------------------------------------------------------
# Basis and AO values
# ----------------------------------------------------------------------------

@dataclasses.dataclass
class Shell:
    center: np.ndarray  # (3,)
    l: int  # 0 (s), 1 (p: x, y, z) or 2 (d: xx, xy, xz, yy, yz, zz), Cartesian
    exponents: np.ndarray
    coefficients: np.ndarray  # contraction coefficients incl. primitive normalisation


def primitive_norm(alpha, l):
    """Normalisation of x^l exp(-alpha r^2) (one Cartesian component)."""
    return (2.0 * alpha / math.pi) ** 0.75 * (4.0 * alpha) ** (0.5 * l)


def cart_components(l):
    """Exponents (i, j, k) of the Cartesian components of angular momentum l in
    pyscf's order: i = l..0, then j = l-i..0, k = l-i-j."""
    return [(i, l - i - k, k) for i in range(l, -1, -1) for k in range(0, l - i + 1)]


def ncart(l):
    return (l + 1) * (l + 2) // 2


def nao_of(shells):
    return sum(ncart(s.l) for s in shells)


def eval_ao(shells, coords, deriv=0):
    """AO values (G, nao) of Cartesian contracted GTOs (pyscf ``eval_gto`` with
    'GTOval_cart', as reached from ``qedft/train/td/eval_gto.py:20-70`` and
    ``qedft/train/td/scf_functions_masked.py:169-173``).  With deriv=1 also
    returns the gradient (3, G, nao)."""
    coords = np.asarray(coords, dtype=np.float64)
    G = coords.shape[0]
    ao = np.zeros((G, nao_of(shells)))
    grad = np.zeros((3, G, nao_of(shells))) if deriv else None
    k = 0
    for s in shells:
        d = coords - s.center[None, :]
        r2 = np.sum(d * d, axis=1)
        e = np.exp(-np.outer(r2, s.exponents))  # (G, nprim)
        rad = e @ s.coefficients
        drad = e @ (-2.0 * s.exponents * s.coefficients)  # (d rad / d r) / r
        for c in cart_components(s.l):
            mono = d[:, 0] ** c[0] * d[:, 1] ** c[1] * d[:, 2] ** c[2]
            ao[:, k] = mono * rad
            if deriv:
                for q in range(3):
                    if c[q] > 0:
                        e_q = list(c)
                        e_q[q] -= 1
                        dm = c[q] * d[:, 0] ** e_q[0] * d[:, 1] ** e_q[1] * d[:, 2] ** e_q[2]
                    else:
                        dm = 0.0
                    grad[q, :, k] = dm * rad + mono * drad * d[:, q]
            k += 1
    return (ao, grad) if deriv else ao


# ----------------------------------------------------------------------------
# numint (LDA)
# ----------------------------------------------------------------------------

def eval_rho(ao, dm):
    """rho_g = sum_ij ao_gi D_ij ao_gj (``qedft/train/td/numint_legacy.py:351-397``,
    LDA branch; ``_dot_ao_dm`` :459-471 and ``_contract_rho`` :475-481)."""
    c0 = ao @ dm
    return np.einsum("gi,gi->g", c0, ao)


def lda_x(rho):
    """Slater exchange: exc = -C rho^(1/3), vrho = 4/3 exc (libxc LDA_X, the
    exchange part of the reference's "LDA,VWN", ``qedft/train/td/rks.py:172``)."""
    rho = np.asarray(rho, dtype=np.float64)
    r13 = np.cbrt(np.maximum(rho, 0.0))
    exc = -SLATER_CX * r13
    return exc, 4.0 / 3.0 * exc


def vwn5_c(rho):
    """VWN correlation, paramagnetic fit 5 (Vosko, Wilk, Nusair, Can. J. Phys. 58,
    1200 (1980); libxc's "VWN" in the reference's "LDA,VWN", ``rks.py:172``):
    (eps_c, v_c = d(rho eps_c)/d rho) in Hartree."""
    rho = np.asarray(rho, dtype=np.float64)
    A, b, c, x0 = 0.0310907, 3.72744, 12.9352, -0.10498
    ok = rho > 1e-30
    r = np.where(ok, rho, 1.0)
    rs = np.cbrt(3.0 / (4.0 * np.pi * r))
    x = np.sqrt(rs)
    X = x * x + b * x + c
    X0 = x0 * x0 + b * x0 + c
    Q = np.sqrt(4.0 * c - b * b)
    t = 2.0 * x + b
    at = np.arctan(Q / t)
    f = b * x0 / X0
    eps = A * (np.log(x * x / X) + 2.0 * b / Q * at
               - f * (np.log((x - x0) ** 2 / X) + 2.0 * (b + 2.0 * x0) / Q * at))
    den = t * t + Q * Q
    de_dx = A * (2.0 / x - t / X - 4.0 * b / den
                 - f * (2.0 / (x - x0) - t / X - 4.0 * (b + 2.0 * x0) / den))
    v = eps - x / 6.0 * de_dx
    return np.where(ok, eps, 0.0), np.where(ok, v, 0.0)


def pbe_x(rho, sigma):
    """PBE exchange, spin-unpolarised (Perdew, Burke, Ernzerhof, PRL 77, 3865
    (1996); libxc's GGA_X_PBE): e = A rho^(4/3) F(s^2), F(u) = 1 + kappa -
    kappa / (1 + mu u / kappa), s = |grad rho| / (2 (3 pi^2)^(1/3) rho^(4/3)).
    Returns (exc per particle, vrho = de/drho, vsigma = de/dsigma)."""
    rho = np.asarray(rho, dtype=np.float64)
    sigma = np.asarray(sigma, dtype=np.float64)
    A = -0.75 * (3.0 / math.pi) ** (1.0 / 3.0)
    kappa, mu = 0.804, 0.2195149727645171
    cs = 1.0 / (4.0 * (3.0 * math.pi ** 2) ** (2.0 / 3.0))
    ok = rho > 1e-14
    r = np.where(ok, rho, 1.0)
    r13 = np.cbrt(r)
    r43 = r * r13
    u = cs * sigma / (r43 * r43)
    den = kappa + mu * u
    F = 1.0 + kappa - kappa * kappa / den
    dF = kappa * kappa * mu / (den * den)
    exc = A * r13 * F
    vr = A * r13 * (4.0 / 3.0 * F - 8.0 / 3.0 * u * dF)
    vs = A * cs * dF / r43
    return np.where(ok, exc, 0.0), np.where(ok, vr, 0.0), np.where(ok, vs, 0.0)


def eval_rho_gga(ao4, dm):
    """(4, G): rho and grad rho (make_rho "GGA", ``numint_legacy.py:180``;
    pyscf eval_rho with c0 = ao0 D, rho_q = 2 sum c0 ao_q)."""
    c0 = ao4[0] @ dm
    out = np.empty((4, ao4.shape[1]))
    out[0] = np.einsum("gi,gi->g", c0, ao4[0])
    for q in range(1, 4):
        out[q] = 2.0 * np.einsum("gi,gi->g", c0, ao4[q])
    return out


def nr_rks_gga(ao4, weights, dm):
    """The GGA branch of ``qedft/train/td/numint_legacy.py:175-198`` with PBE
    exchange: wv0 = 0.5 w vrho, wv_q = 2 w vsigma drho/dq (``_rks_gga_wv0``),
    aow = sum_n wv_n ao_n (``_scale_ao``), vmat = ao0^T aow + transpose (:337)."""
    rho = eval_rho_gga(ao4, dm)
    sigma = np.sum(rho[1:] ** 2, axis=0)
    exc, vrho, vsigma = pbe_x(rho[0], sigma)
    den = rho[0] * weights
    wv = np.empty((4, rho.shape[1]))
    wv[0] = 0.5 * weights * vrho
    wv[1:] = 2.0 * weights * vsigma * rho[1:]
    aow = np.einsum("npi,np->pi", ao4, wv)
    vmat = ao4[0].T @ aow
    return den.sum(), float(np.dot(den, exc)), vmat + vmat.T


def nr_rks_lda(ao, weights, dm, vwn=False):
    """(nelec, excsum, vmat) of ``qedft/train/td/numint_legacy.py:122-164,337``:
    aow = 0.5 * w * vrho * ao; vmat = ao^T aow; vmat += vmat^T."""
    rho = eval_rho(ao, dm)
    exc, vrho = lda_x(rho)
    if vwn:
        ec, vc = vwn5_c(rho)
        exc, vrho = exc + ec, vrho + vc
    den = rho * weights
    nelec = den.sum()
    excsum = np.dot(den, exc)
    aow = ao * (0.5 * weights * vrho)[:, None]
    vmat = ao.T @ aow
    return nelec, excsum, vmat + vmat.T


# ----------------------------------------------------------------------------
# Neural XC (local MLP)
# ----------------------------------------------------------------------------
def _gelu(x):
    """flax/jax gelu, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))."""
    c = x.dtype.type(np.sqrt(2.0 / np.pi))
    a = x.dtype.type(0.044715)
    half = x.dtype.type(0.5)
    one = x.dtype.type(1.0)
    t = np.tanh(c * (x + a * x ** 3))
    d = half * (one + t) + half * x * (one - t * t) * c * (one + x.dtype.type(3.0) * a * x * x)
    return half * x * (one + t), d


def nn_xc_local(flat, rho, scale=1e-2, dtype=np.float64):
    """(exc, vrho) of ``get_exc_and_vrho`` (``qedft/train/td/xc.py:12-47``) for the
    local MLP of ``qedft/train/td/trainer_legacy_no_jit.py:56-62, 98-107``:
    exc_g = -scale swish(w3 . gelu(gelu(rho_g w1 + b1) W2 + b2) + b3) and
    vrho_g = d exc_g / d rho_g (the vjp with ones of a per-point map), evaluated
    in ``dtype``.  ``flat`` = (w1, b1, W2 (in, out), b2, w3, b3)."""
    flat = np.asarray(flat, dtype)
    H = int(round((-3 + np.sqrt(9 + 4 * (flat.size - 1))) / 2))
    w1, b1 = flat[:H], flat[H:2 * H]
    W2 = flat[2 * H:2 * H + H * H].reshape(H, H)
    o = 2 * H + H * H
    b2, w3, b3 = flat[o:o + H], flat[o + H:o + 2 * H], flat[o + 2 * H]
    x = np.asarray(rho, dtype)[:, None]
    h1, d1 = _gelu(x * w1[None, :] + b1[None, :])
    z2 = h1 @ W2 + b2[None, :]
    h2, d2 = _gelu(z2)
    z3 = h2 @ w3 + b3
    sg = 1 / (1 + np.exp(-z3))
    s = dtype(scale)
    exc = -s * z3 * sg
    dz3 = -s * sg * (1 + z3 * (1 - sg))
    dz2 = (dz3[:, None] * w3[None, :]) * d2
    dh1 = dz2 @ W2.T
    vrho = (dh1 * d1) @ w1
    return exc, vrho


def nn_xc_global(flat, rho, hidden, scale=1e-2, dtype=np.float64):
    """(exc, vrho) of ``exc_and_vrho_global`` (``qedft/train/td/trainer_legacy_no_jit.py:46-53``):
    the density vector (G) is one input of the MLP [H, H, 1]; exc is the scalar sum of
    its output, vrho = d exc / d rho.  ``flat`` = (W1 (G, H), b1, W2, b2, w3, b3)."""
    flat = np.asarray(flat, dtype)
    x = np.asarray(rho, dtype)
    G, H = x.size, int(hidden)
    W1 = flat[:G * H].reshape(G, H)
    o = G * H
    b1 = flat[o:o + H]
    W2 = flat[o + H:o + H + H * H].reshape(H, H)
    o += H + H * H
    b2, w3, b3 = flat[o:o + H], flat[o + H:o + 2 * H], flat[o + 2 * H]
    h1, d1 = _gelu(x @ W1 + b1)
    h2, d2 = _gelu(h1 @ W2 + b2)
    z3 = h2 @ w3 + b3
    sg = 1 / (1 + np.exp(-z3))
    s = dtype(scale)
    exc = -s * z3 * sg
    dz3 = -s * sg * (1 + z3 * (1 - sg))
    dz2 = dz3 * w3 * d2
    dz1 = (W2 @ dz2) * d1
    return exc, W1 @ dz1


def nr_rks_nn(ao, weights, dm, flat, scale=1e-2, dtype=np.float64, hidden=None):
    """``nr_rks_lda`` with the neural functional in place of the LDA exchange: the
    local network (exc per point), or with ``hidden`` the global network, whose
    scalar output is added as the XC energy (``numint_legacy.py:311-333``)."""
    rho = eval_rho(ao, dm)
    den = rho * weights
    nelec = den.sum()
    if hidden is not None:
        exc, vrho = nn_xc_global(flat, rho, hidden, scale, dtype)
        aow = ao * (0.5 * weights * np.asarray(vrho, np.float64))[:, None]
        vmat = ao.T @ aow
        return nelec, float(exc), vmat + vmat.T
    exc, vrho = nn_xc_local(flat, rho, scale, dtype)
    exc, vrho = np.asarray(exc, np.float64), np.asarray(vrho, np.float64)
    excsum = np.dot(den, exc)
    aow = ao * (0.5 * weights * vrho)[:, None]
    vmat = ao.T @ aow
    return nelec, excsum, vmat + vmat.T


# ----------------------------------------------------------------------------
# Generalized eigensolver
# ----------------------------------------------------------------------------

def generalized_eigh(A, B, eps=1e-12):
    """``qedft/train/td/generalized_eigensolver.py:264-330``: symmetrise, shift B
    if its smallest eigenvalue is below eps, Cholesky, C = L^-1 A L^-T, eigh(C),
    V = L^-T U."""
    import scipy.linalg as sla

    A = 0.5 * (A + A.T)
    B = 0.5 * (B + B.T)
    lam_min = np.linalg.eigvalsh(B).min()
    if lam_min < eps:
        B = B + (eps - lam_min) * np.eye(B.shape[0])
    L = np.linalg.cholesky(B)
    Y = sla.solve_triangular(L, A, lower=True)
    C = sla.solve_triangular(L, Y.T, lower=True).T
    C = 0.5 * (C + C.T)
    w, U = np.linalg.eigh(C)
    V = sla.solve_triangular(L.T, U, lower=False)
    return w, V


def masked_generalized_eigh(fock, s1e, mask):
    """``qedft/train/td/generalized_eigensolver_masked.py:19-89``."""
    mask = np.asarray(mask, dtype=bool)
    n = fock.shape[0]
    m2 = mask[:, None] & mask[None, :]
    eye = np.eye(n, dtype=bool)
    f = np.where(m2, fock, 0.0) + np.where(~mask[:, None] & eye, 1e-12, 0.0)
    s = np.where(m2, s1e, np.where(~mask[:, None] & eye, 1e-12, 0.0))
    w, v = generalized_eigh(f, s)
    key = np.where(mask, w, 1e12)  # mask indexes basis functions; reference uses it per eigenvalue slot
    order = np.argsort(key, kind="stable")
    w = w[order] * mask[order]
    v = np.where(m2[:, order], v[:, order], 0.0)
    return w, v


# ----------------------------------------------------------------------------
# Occupations, density matrix, DIIS, energies
# ----------------------------------------------------------------------------

# ----------------------------------------------------------------------------
# Fractional (Fermi-Dirac) occupations, qedft/train/td/fermi.py
# ----------------------------------------------------------------------------

def fermi_function4entropy(energy, mu, theta):
    """1 / (1 + exp((e - mu) / theta)) (``qedft/train/td/fermi.py:13-29``)."""
    with np.errstate(over="ignore"):  # exp -> inf gives the limit 0
        return 1.0 / (1.0 + np.exp((np.asarray(energy, np.float64) - mu) / theta))


def fermi_function(energy, mu, theta):
    """2 / (1 + exp((e - mu) / theta)), restricted occupation (``fermi.py:32-50``)."""
    return 2.0 * fermi_function4entropy(energy, mu, theta)


def _fermi_count(mu, mo_energy, theta):
    """F = sum occ and its first two mu-derivatives."""
    s = fermi_function4entropy(mo_energy, mu, theta)
    q = s * (1.0 - s)
    return (float(np.sum(2.0 * s)), float(np.sum(2.0 * q)) / theta,
            float(np.sum(2.0 * q * (1.0 - 2.0 * s))) / (theta * theta))


def loss_fermi_function(mu, mo_energy, n, theta):
    """(N - sum occ)^2 (``fermi.py:53-78``)."""
    return (n - _fermi_count(mu, mo_energy, theta)[0]) ** 2


def _loss_derivatives(mu, mo_energy, n, theta):
    """d/dmu and d2/dmu2 of the loss (what jax.grad gives at ``fermi.py:142-143``)."""
    f, f1, f2 = _fermi_count(mu, mo_energy, theta)
    r = n - f
    return -2.0 * r * f1, 2.0 * f1 * f1 - 2.0 * r * f2


def make_occ_fermi(mu, mo_energy, theta):
    """``fermi.py:81-100``."""
    return fermi_function(mo_energy, mu, theta)


def entropy(f):
    """f ln f + (1 - f) ln(1 - f) (``fermi.py:103-115``), with 0 ln 0 = 0 (the
    reference's expression evaluates to NaN where an occupation is exactly 0 or 1)."""
    f = np.asarray(f, np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        a = np.where(f > 0.0, f * np.log(np.where(f > 0.0, f, 1.0)), 0.0)
        b = np.where(f < 1.0, (1.0 - f) * np.log(np.where(f < 1.0, 1.0 - f, 1.0)), 0.0)
    return a + b


def etropic_energy_contribution(mu, mo_energy, theta):
    """theta sum 2 entropy(f) (``fermi.py:118-139``)."""
    return float(theta * np.sum(2.0 * entropy(fermi_function4entropy(mo_energy, mu, theta))))


def optimize_fermi_occupations(mo_energy, n_electrons, theta=0.04, mu_initial=None,
                               mu_shift=0.001, step_grad=0.6, max_steps=100, tol=1e-9):
    """Damped Newton on the chemical potential, stopping once the loss is below
    ``tol``; ValueError if it ends above 1e-2 (``fermi.py:145-219``)."""
    e = np.asarray(mo_energy, np.float64)
    mu = float(e[0] + mu_shift) if mu_initial is None else float(mu_initial)
    loss = 100.0
    for _ in range(int(max_steps)):
        g, gg = _loss_derivatives(mu, e, n_electrons, theta)
        safe = 1e-10 * np.sign(gg) if abs(gg) < 1e-10 else gg
        mu = mu - step_grad * g / safe
        loss = loss_fermi_function(mu, e, n_electrons, theta)
        if loss < tol:
            break
    if loss > 1e-2:
        raise ValueError(f"Fermi occupation optimization failed: loss={loss}.")
    return make_occ_fermi(mu, e, theta), etropic_energy_contribution(mu, e, theta), mu, loss


def get_fractional_occupations(mo_energy, n_electrons, frac_mo_occ=1, frac_theta=0.04,
                               frac_mu=None, frac_mu_shift=0.001, frac_step_grad=0.6,
                               frac_max_steps=100):
    """``fermi.py:222-298``: 1 -> Fermi-Dirac, an array -> given, None -> aufbau
    with a fractional remainder."""
    e = np.asarray(mo_energy, np.float64)
    if isinstance(frac_mo_occ, (int, float)) and not isinstance(frac_mo_occ, bool) \
            and frac_mo_occ == 1:
        return optimize_fermi_occupations(e, n_electrons, frac_theta, frac_mu, frac_mu_shift,
                                          frac_step_grad, frac_max_steps)
    if isinstance(frac_mo_occ, np.ndarray):
        return frac_mo_occ, 0.0, None, None
    if frac_mo_occ is None:
        occ = np.zeros_like(e)
        rem = float(n_electrons)
        for i in range(e.size):
            if rem >= 2.0:
                occ[i], rem = 2.0, rem - 2.0
            elif rem > 0.0:
                occ[i], rem = rem, 0.0
            else:
                break
        return occ, 0.0, None, None
    raise ValueError(f"frac_mo_occ={frac_mo_occ} not implemented")


def get_fractional_occupations_jax(mo_energy, n_electrons, theta, frac_mu, frac_mu_shift,
                                   frac_step_grad, frac_max_steps):
    """Fixed number of damped Newton steps, min(frac_max_steps, 100), no early
    stop (``fermi.py:301-390``)."""
    e = np.asarray(mo_energy, np.float64)
    mu = float(e[0] + frac_mu_shift) if frac_mu is None else float(frac_mu)
    loss = 1.0
    for _ in range(min(int(frac_max_steps), 100)):
        g, gg = _loss_derivatives(mu, e, n_electrons, theta)
        safe = np.sign(gg) * max(abs(gg), 1e-10)
        mu = mu - frac_step_grad * g / safe
        loss = loss_fermi_function(mu, e, n_electrons, theta)
    return (make_occ_fermi(mu, e, theta), etropic_energy_contribution(mu, e, theta), mu, loss)


def get_fractional_occupations_jax_stable(mo_energy, n_electrons, theta, frac_mu, frac_mu_shift,
                                          frac_step_grad, frac_max_steps):
    """Newton from the HOMO/LUMO midpoint; if the electron count misses by 1e-2
    or more, 10 fixed-point steps at theta = 0.01 from the midpoint instead
    (``fermi.py:393-497``).  Loss reported as 0."""
    e = np.asarray(mo_energy, np.float64)
    n = e.size
    n_double = int(np.floor(n_electrons / 2.0))
    rem = n_electrons - 2.0 * n_double
    # jnp indexing clamps out-of-range indices (fermi.py:422-427): more than
    # 2n electrons take the highest orbital for both
    homo = min(max(n_double - 1, 0), n - 1)
    lumo = max(min(n_double + (1 if rem > 0 else 0), n - 1), 0)
    default_mu = 0.5 * (e[homo] + e[lumo])
    mu = default_mu if frac_mu is None else float(frac_mu)
    for _ in range(min(int(frac_max_steps), 100)):
        g, gg = _loss_derivatives(mu, e, n_electrons, theta)
        safe = 1e-10 if abs(gg) < 1e-10 else gg
        mu = mu - frac_step_grad * g / safe
    occ = make_occ_fermi(mu, e, theta)
    if abs(np.sum(occ) - n_electrons) < 1e-2:
        return occ, etropic_energy_contribution(mu, e, theta), mu, 0.0
    small = 0.01
    mu_fb = default_mu
    for _ in range(10):
        mu_fb = mu_fb - 0.1 * (np.sum(make_occ_fermi(mu_fb, e, small)) - n_electrons)
    return (make_occ_fermi(mu_fb, e, small), etropic_energy_contribution(mu_fb, e, small),
            mu_fb, 0.0)


def get_occ(nelectron, mo_energy):
    """Aufbau, 2 electrons in each of the lowest Ne/2 orbitals
    (``qedft/train/td/scf_functions_masked.py:176-186``)."""
    e_idx = np.argsort(mo_energy, kind="stable")
    occ_sorted = np.where(np.arange(mo_energy.size) < nelectron // 2, 2.0, 0.0)
    occ = np.empty_like(occ_sorted)
    occ[e_idx] = occ_sorted
    return occ


def make_rdm1(mo_coeff, mo_occ):
    """D = C_occ diag(occ) C_occ^H over the orbitals with occ > 0
    (``qedft/train/td/hf.py:303-308``)."""
    mo_occ = np.asarray(mo_occ)
    sel = mo_occ > 0
    mocc = np.asarray(mo_coeff)[:, sel]
    # the unoccupied columns are dropped, not weighted by 0: a non-finite
    # entry there (padding of a masked eigensolve) does not reach D
    return (mocc * mo_occ[sel]) @ mocc.conj().T


class DIIS:
    """CDIIS restated from ``qedft/train/td/jax_diis.py:10-134``."""

    def __init__(self, max_vec=8, min_vecs=2):
        self.max_vec, self.min_vecs = max_vec, min_vecs
        self.errs, self.focks = [], []

    @staticmethod
    def error(fock, dm, ovlp):
        return fock @ (dm @ ovlp) - ovlp @ (dm @ fock)

    def update(self, fock, dm, ovlp):
        self.errs.append(self.error(fock, dm, ovlp).ravel())
        self.focks.append(fock.ravel())
        if len(self.errs) > self.max_vec:
            self.errs = self.errs[-self.max_vec:]
            self.focks = self.focks[-self.max_vec:]
        n = len(self.errs)
        if n < self.min_vecs:
            return self.focks[-1].reshape(fock.shape)
        B = np.zeros((n + 1, n + 1))
        B[0, 1:] = -1.0
        B[1:, 0] = -1.0
        E = np.array(self.errs)
        B[1:, 1:] = E @ E.T
        B[np.diag_indices(n + 1)] += 1e-14
        rhs = np.zeros(n + 1)
        rhs[0] = -1.0
        c = np.linalg.solve(B, rhs)[1:]
        return (c @ np.array(self.focks)).reshape(fock.shape)


def coulomb_lowrank(factors, dm):
    """J_ij = sum_kl (ij|kl) D_kl with (ij|kl) = sum_P B_P,ij B_P,kl."""
    c = np.einsum("pij,ij->p", factors, dm)
    return np.einsum("p,pij->ij", c, factors)


def energy_tot(dm, h1e, J, exc, e_nuc):
    """``qedft/train/td/scf_functions_masked.py:162-166``."""
    return float(np.einsum("ij,ji->", dm, h1e) + 0.5 * np.einsum("ij,ij->", dm, J) + exc + e_nuc)


def orbital_gradient_norm(mo_coeff, mo_occ, fock):
    """|g|, g = 2 C_vir^T F C_occ: pyscf's RHF ``get_grad`` as the reference's
    loop calls it (``qedft/train/td/hf.py:81-84``; occupied = mo_occ > 0)."""
    occ = np.asarray(mo_occ) > 0
    g = 2.0 * mo_coeff[:, ~occ].T @ fock @ mo_coeff[:, occ]
    return float(np.linalg.norm(g))


def scf(mol, max_cycle=30, diis_max_vec=8, diis_start_cycle=1, nn=None, vwn=False, fermi=None,
        gga=False, stop=None):
    """Fixed-cycle SCF of ``qedft/train/td/scf_functions_masked.py:907-967`` with
    the low-rank Coulomb model and the LDA exchange, or with ``nn = (flat,
    scale, dtype)`` the neural functional.  ``fermi`` (a dict: theta, mode
    "stable" (default) / "jax" / "optimize", max_steps, step_grad, mu_shift, mu) replaces
    the aufbau occupations by Fermi-Dirac ones (``qedft/train/td/fermi.py``);
    the per-cycle entropic energies are then returned as a fourth value.
    ``gga=True`` uses the GGA branch with PBE exchange (``nr_rks_gga``).
    ``stop = (conv_tol, conv_tol_grad)``: the loop of ``qedft/train/td/hf.py:47-110``
    instead, which stops at the first cycle with |E - E_last| < conv_tol and
    |g| < conv_tol_grad (E_last of cycle 0 = the initial guess's energy); it
    returns a dict (e_tot, dm, mo_energy, mo_occ, converged, cycles, energies,
    grad_norms)."""
    ao, w = mol.ao, mol.weights
    if gga:
        ao = eval_ao(mol.shells, mol.coords, deriv=1)
        ao = np.concatenate([ao[0][None], ao[1]], axis=0)

        def rks(ao, w, dm):
            return nr_rks_gga(ao, w, dm)
    elif nn is None:
        def rks(ao, w, dm):
            return nr_rks_lda(ao, w, dm, vwn=vwn)
    else:
        def rks(ao, w, dm):
            return nr_rks_nn(ao, w, dm, *nn)
    s1e, h1e = mol.s1e, mol.h1e

    def occupations(mo_e):
        if fermi is None:
            return get_occ(mol.nelectron, mo_e), 0.0
        args = (mo_e, float(mol.nelectron), fermi.get("theta", 0.04), fermi.get("mu"),
                fermi.get("mu_shift", 0.001), fermi.get("step_grad", 0.6),
                fermi.get("max_steps", 100))
        mode = fermi.get("mode", "stable")
        if mode == "jax":
            occ, entr, _, _ = get_fractional_occupations_jax(*args)
        elif mode == "stable":
            occ, entr, _, _ = get_fractional_occupations_jax_stable(*args)
        else:
            occ, entr, _, _ = optimize_fermi_occupations(mo_e, float(mol.nelectron), args[2],
                                                         args[3], args[4], args[5], args[6])
        return occ, entr

    e0, c0 = generalized_eigh(h1e, s1e)
    dm = make_rdm1(c0, occupations(e0)[0])
    J = coulomb_lowrank(mol.eri_factors, dm)
    _, exc, vxc = rks(ao, w, dm)
    vhf = J + vxc
    e_last = energy_tot(dm, h1e, J, exc, mol.energy_nuc)
    diis = DIIS(diis_max_vec)
    energies, entropic, gnorms = [], [], []
    converged = False
    for cycle in range(max_cycle):
        fock = h1e + vhf
        if cycle >= diis_start_cycle:
            fock = diis.update(fock, dm, s1e)
        mo_e, mo_c = generalized_eigh(fock, s1e)
        occ, entr = occupations(mo_e)
        entropic.append(entr)
        dm = make_rdm1(mo_c, occ)
        J = coulomb_lowrank(mol.eri_factors, dm)
        _, exc, vxc = rks(ao, w, dm)
        vhf = J + vxc
        energies.append(energy_tot(dm, h1e, J, exc, mol.energy_nuc))
        if stop is not None:
            gnorms.append(orbital_gradient_norm(mo_c, occ, h1e + vhf))
            if abs(energies[-1] - e_last) < stop[0] and gnorms[-1] < stop[1]:
                converged = True
                break
            e_last = energies[-1]
    if stop is not None:
        return {"e_tot": energies[-1], "dm": dm, "mo_energy": mo_e, "mo_occ": occ,
                "converged": converged, "cycles": len(energies),
                "energies": np.array(energies), "grad_norms": np.array(gnorms)}
    if fermi is not None:
        return np.array(energies), dm, mo_e, np.array(entropic)
    return np.array(energies), dm, mo_e


# ----------------------------------------------------------------------------
# Molecular grids (pyscf gen_grid.Grids with becke_scheme = stratmann, as the
# reference builds them at qedft/data_io/td/dataset_generation.py:139-142)
# ----------------------------------------------------------------------------

_BRAGG = {1: 0.35, 2: 1.40, 3: 1.45, 4: 1.05, 5: 0.85, 6: 0.70, 7: 0.65, 8: 0.60, 9: 0.50,
          10: 1.50}
_XI = {1: 0.8, 2: 0.9, 3: 1.8, 4: 1.4, 5: 1.3, 6: 1.1, 7: 0.9, 8: 0.9, 9: 0.9, 10: 0.9}
_RAD = ((10, 30, 40, 50, 60, 70, 80, 90, 100, 200), (15, 40, 60, 75, 90, 105, 120, 135, 150, 200))
_ANG = (6, 8, 10, 12, 14, 16, 18, 20, 22, 24)


def radial_m4(n, xi):
    """Treutler-Ahlrichs M4 mapping r = xi/ln2 (1+x)^0.6 ln(2/(1-x)) on the
    Chebyshev nodes of the second kind x_i = cos(i pi/(n+1)) (J. Chem. Phys.
    102, 346 (1995)); weights r^2 dr with dr = pi/(n+1) sin(theta_i) r'(x_i)."""
    th = np.arange(1, n + 1) * math.pi / (n + 1)
    x = np.cos(th)
    r = xi / math.log(2.0) * (1.0 + x) ** 0.6 * np.log(2.0 / (1.0 - x))
    drdx = xi / math.log(2.0) * ((0.6 * (1.0 + x) ** -0.4) * np.log(2.0 / (1.0 - x))
                                 + (1.0 + x) ** 0.6 / (1.0 - x))
    dr = math.pi / (n + 1) * np.sin(th) * drdx
    return r[::-1], (r * r * dr)[::-1]


def angular_rule(n_theta):
    """Gauss-Legendre in cos(theta) x 2 n_theta uniform phi (offset half a step)."""
    t, wt = np.polynomial.legendre.leggauss(n_theta)
    n_phi = 2 * n_theta
    phi = (np.arange(n_phi) + 0.5) * 2.0 * math.pi / n_phi
    st = np.sqrt(1.0 - t * t)
    u = np.stack([np.outer(st, np.cos(phi)).ravel(), np.outer(st, np.sin(phi)).ravel(),
                  np.repeat(t, n_phi)], axis=1)
    return u, np.repeat(wt, n_phi) * 2.0 * math.pi / n_phi


def switch_g(mu, scheme="stratmann"):
    """Stratmann's polynomial (a = 0.64; CPL 257, 213 (1996)) or Becke's three
    iterations of 1.5 m - 0.5 m^3 (J. Chem. Phys. 88, 2547 (1988))."""
    mu = np.asarray(mu, dtype=np.float64)
    if scheme == "stratmann":
        a = 0.64
        m = mu / a
        m2 = m * m
        g = m * (35.0 + m2 * (-35.0 + m2 * (21.0 - 5.0 * m2))) / 16.0
        return np.where(mu <= -a, -1.0, np.where(mu >= a, 1.0, g))
    g = mu
    for _ in range(3):
        g = 1.5 * g - 0.5 * g ** 3
    return g


def becke_grid(charges, positions, level=3, scheme="stratmann", size_adjust=True):
    """(coords (G, 3), weights (G)): atom-centred M4 x product grids, Becke's
    partition with his size adjustment (a_bc from the Bragg-Slater radius ratio,
    clipped to 1/2) and the chosen switching function; points packed atom by
    atom, radial-major."""
    z = [int(q) for q in charges]
    xyz = np.asarray(positions, dtype=np.float64).reshape(-1, 3)
    u, wa = angular_rule(_ANG[level])
    pts, wts = [], []
    for a, za in enumerate(z):
        r, wr = radial_m4(_RAD[0 if za <= 2 else 1][level], _XI.get(za, 1.0))
        pts.append((xyz[a][None, None, :] + r[:, None, None] * u[None, :, :]).reshape(-1, 3))
        wts.append(np.outer(wr, wa).ravel())
    R = np.array([_BRAGG.get(q, 1.0) for q in z])
    chi = R[:, None] / R[None, :]
    uu = (chi - 1.0) / (chi + 1.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        adj = np.clip(np.where(np.abs(uu) > 0, uu / (uu * uu - 1.0), 0.0), -0.5, 0.5)
    coords, weights = [], []
    nat = len(z)
    for a in range(nat):
        x = pts[a]
        if nat == 1:
            coords.append(x)
            weights.append(wts[a])
            continue
        d = np.linalg.norm(x[:, None, :] - xyz[None, :, :], axis=2)  # (G_a, natom)
        P = np.ones((x.shape[0], nat))
        for b in range(nat):
            for c in range(nat):
                if b == c:
                    continue
                mu = (d[:, b] - d[:, c]) / np.linalg.norm(xyz[b] - xyz[c])
                nu = mu + adj[b, c] * (1.0 - mu * mu) if size_adjust else mu
                P[:, b] *= 0.5 * (1.0 - switch_g(nu, scheme))
        coords.append(x)
        weights.append(wts[a] * P[:, a] / P.sum(axis=1))
    return np.concatenate(coords), np.concatenate(weights)


# ----------------------------------------------------------------------------
# Gaussian integrals (McMurchie-Davidson; Helgaker, Joergensen, Olsen,
# "Molecular Electronic-Structure Theory", ch. 9) for Cartesian s, p and d
# primitives: what pyscf's libcint provides to the reference (int1e_ovlp,
# int1e_kin, int1e_nuc, int3c2e, int2c2e for density fitting,
# qedft/train/td/hf.py:425-449 via pyscfad df_jk).
# ----------------------------------------------------------------------------

def boys(n, T):
    """F_n(T) = int_0^1 t^(2n) exp(-T t^2) dt, through the regularised lower
    incomplete gamma function: Gamma(n+1/2) P(n+1/2, T) / (2 T^(n+1/2))."""
    from scipy.special import gamma, gammainc

    T = float(T)
    if T < 1e-12:
        return 1.0 / (2 * n + 1) - T / (2 * n + 3)
    return gamma(n + 0.5) * gammainc(n + 0.5, T) / (2.0 * T ** (n + 0.5))


def _hermite_e(i, j, a, b, XAB):
    """E^{ij}_t, t = 0..i+j, for one Cartesian direction (the Gaussian product
    of exponents a, b separated by XAB = A - B)."""
    p = a + b
    mu = a * b / p
    XPA = -b / p * XAB
    XPB = a / p * XAB
    E = {(0, 0): np.array([math.exp(-mu * XAB * XAB)])}

    def get(ii, jj):
        if (ii, jj) in E:
            return E[(ii, jj)]
        if ii > 0:
            prev = get(ii - 1, jj)
            X = XPA
        else:
            prev = get(ii, jj - 1)
            X = XPB
        n = ii + jj
        out = np.zeros(n + 1)
        for t in range(n + 1):
            v = X * (prev[t] if t < prev.size else 0.0)
            if t >= 1:
                v += prev[t - 1] / (2.0 * p)
            if t + 1 < prev.size:
                v += (t + 1) * prev[t + 1]
            out[t] = v
        E[(ii, jj)] = out
        return out

    return get(i, j)


def _hermite_r(L, p, X, Y, Z):
    """R_{tuv} (t+u+v <= L) of the Hermite Coulomb integrals for exponent p and
    the vector (X, Y, Z) between the Hermite centres."""
    T = p * (X * X + Y * Y + Z * Z)
    R = {}

    def r(n, t, u, v):
        key = (n, t, u, v)
        if key in R:
            return R[key]
        if t < 0 or u < 0 or v < 0:
            return 0.0
        if t == u == v == 0:
            val = (-2.0 * p) ** n * boys(n, T)
        elif t > 0:
            val = (t - 1) * r(n + 1, t - 2, u, v) + X * r(n + 1, t - 1, u, v)
        elif u > 0:
            val = (u - 1) * r(n + 1, t, u - 2, v) + Y * r(n + 1, t, u - 1, v)
        else:
            val = (v - 1) * r(n + 1, t, u, v - 2) + Z * r(n + 1, t, u, v - 1)
        R[key] = val
        return val

    return lambda t, u, v: r(0, t, u, v)


def _self_e(l, g):
    """Hermite expansion of x^l exp(-g x^2) about its own centre (E_t, t <= l)."""
    return _hermite_e(l, 0, g, 0.0, 0.0)


def _prims(shell):
    return list(zip(shell.exponents, shell.coefficients))


def int1e(shells, charges, positions):
    """(S, T, V): overlap, kinetic and nuclear attraction -sum_C Z_C / |r - C|
    over the contracted Cartesian shells."""
    n = nao_of(shells)
    S, T, V = np.zeros((n, n)), np.zeros((n, n)), np.zeros((n, n))
    offs = np.cumsum([0] + [ncart(s.l) for s in shells])
    pos = np.asarray(positions, dtype=np.float64).reshape(-1, 3)
    for ia, A in enumerate(shells):
        for ib, B in enumerate(shells):
            AB = A.center - B.center
            for a, ca in _prims(A):
                for b, cb in _prims(B):
                    p = a + b
                    P = (a * A.center + b * B.center) / p
                    for ka, la in enumerate(cart_components(A.l)):
                        for kb, lb in enumerate(cart_components(B.l)):
                            Ed = [[_hermite_e(la[d], j, a, b, AB[d]) for j in range(lb[d] + 3)]
                                  for d in range(3)]
                            s1 = [Ed[d][lb[d]][0] * math.sqrt(math.pi / p) for d in range(3)]

                            def sij(d, j):
                                return (Ed[d][j][0] * math.sqrt(math.pi / p)) if j >= 0 else 0.0

                            t1 = []
                            for d in range(3):
                                j = lb[d]
                                t1.append(-0.5 * (j * (j - 1) * sij(d, j - 2)
                                                  - 2.0 * b * (2 * j + 1) * sij(d, j)
                                                  + 4.0 * b * b * sij(d, j + 2)))
                            i, j = offs[ia] + ka, offs[ib] + kb
                            cc = ca * cb
                            S[i, j] += cc * s1[0] * s1[1] * s1[2]
                            T[i, j] += cc * (t1[0] * s1[1] * s1[2] + s1[0] * t1[1] * s1[2]
                                             + s1[0] * s1[1] * t1[2])
                            Eab = [Ed[d][lb[d]] for d in range(3)]
                            for zc, C in zip(charges, pos):
                                PC = P - C
                                Rf = _hermite_r(la[0] + lb[0] + la[1] + lb[1] + la[2] + lb[2], p,
                                                *PC)
                                acc = 0.0
                                for t in range(Eab[0].size):
                                    for u in range(Eab[1].size):
                                        for v in range(Eab[2].size):
                                            acc += Eab[0][t] * Eab[1][u] * Eab[2][v] * Rf(t, u, v)
                                V[i, j] -= cc * zc * 2.0 * math.pi / p * acc
    return S, T, V


def int3c2e(shells, aux):
    """(naux, n, n): (ij|P) over AO shells i, j and auxiliary shells P."""
    n, na = nao_of(shells), nao_of(aux)
    out = np.zeros((na, n, n))
    offs = np.cumsum([0] + [ncart(s.l) for s in shells])
    aoffs = np.cumsum([0] + [ncart(s.l) for s in aux])
    for ia, A in enumerate(shells):
        for ib, B in enumerate(shells):
            AB = A.center - B.center
            for ic, Cs in enumerate(aux):
                for a, ca in _prims(A):
                    for b, cb in _prims(B):
                        p = a + b
                        P = (a * A.center + b * B.center) / p
                        for g, cg in _prims(Cs):
                            al = p * g / (p + g)
                            pre = 2.0 * math.pi ** 2.5 / (p * g * math.sqrt(p + g))
                            PC = P - Cs.center
                            for ka, la in enumerate(cart_components(A.l)):
                                for kb, lb in enumerate(cart_components(B.l)):
                                    Eab = [_hermite_e(la[d], lb[d], a, b, AB[d]) for d in range(3)]
                                    for kc, lc in enumerate(cart_components(Cs.l)):
                                        # a single Gaussian about its own centre
                                        Ec = [_self_e(lc[d], g) for d in range(3)]
                                        L = sum(la) + sum(lb) + sum(lc)
                                        Rf = _hermite_r(L, al, *PC)
                                        acc = 0.0
                                        for t in range(Eab[0].size):
                                            for u in range(Eab[1].size):
                                                for v in range(Eab[2].size):
                                                    e1 = Eab[0][t] * Eab[1][u] * Eab[2][v]
                                                    for tt in range(Ec[0].size):
                                                        for uu in range(Ec[1].size):
                                                            for vv in range(Ec[2].size):
                                                                acc += (e1 * (-1) ** (tt + uu + vv)
                                                                        * Ec[0][tt] * Ec[1][uu]
                                                                        * Ec[2][vv]
                                                                        * Rf(t + tt, u + uu, v + vv))
                                        out[aoffs[ic] + kc, offs[ia] + ka, offs[ib] + kb] += (
                                            ca * cb * cg * pre * acc)
    return out


def int2c2e(aux):
    """(naux, naux): (P|Q) over auxiliary shells."""
    na = nao_of(aux)
    out = np.zeros((na, na))
    aoffs = np.cumsum([0] + [ncart(s.l) for s in aux])
    for ia, A in enumerate(aux):
        for ib, B in enumerate(aux):
            for a, ca in _prims(A):
                for b, cb in _prims(B):
                    al = a * b / (a + b)
                    pre = 2.0 * math.pi ** 2.5 / (a * b * math.sqrt(a + b))
                    AB = A.center - B.center
                    for ka, la in enumerate(cart_components(A.l)):
                        for kb, lb in enumerate(cart_components(B.l)):
                            Ea = [_self_e(la[d], a) for d in range(3)]
                            Eb = [_self_e(lb[d], b) for d in range(3)]
                            Rf = _hermite_r(sum(la) + sum(lb), al, *AB)
                            acc = 0.0
                            for t in range(Ea[0].size):
                                for u in range(Ea[1].size):
                                    for v in range(Ea[2].size):
                                        for tt in range(Eb[0].size):
                                            for uu in range(Eb[1].size):
                                                for vv in range(Eb[2].size):
                                                    acc += (Ea[0][t] * Ea[1][u] * Ea[2][v]
                                                            * (-1) ** (tt + uu + vv) * Eb[0][tt]
                                                            * Eb[1][uu] * Eb[2][vv]
                                                            * Rf(t + tt, u + uu, v + vv))
                            out[aoffs[ia] + ka, aoffs[ib] + kb] += ca * cb * pre * acc
    return out
