"""Numerical integration pieces of the 3D Kohn-Sham path on the GPU.

Mirrors ``qedft/train/td/numint_legacy.py``: ``eval_ao`` (AO values),
``eval_rho`` (:351-397), ``nr_rks`` (:122-348, LDA branch :148-164 with the
``vmat + vmat^T`` symmetrisation of :337).  Arrays are torch CUDA tensors
(float64, row-major); every call runs the kernels of ``include/qex_td.h``.
"""

from __future__ import annotations

import numpy as np

from .. import _native as N
from . import _lib


def _dev(a, dtype=None):
    torch = N.require_cuda()
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda", dtype=dtype or a.dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda", dtype=dtype)


def eval_ao(mol, coords=None):
    """(G, nao) AO values of ``mol``'s Cartesian contracted shells on ``coords``."""
    torch = N.require_cuda()
    L = _lib.lib()
    coords = _dev(mol.coords if coords is None else coords, torch.float64)
    centers, l, poff, aoff, ex, co = mol.shell_arrays()
    G = coords.shape[0]
    ao = torch.empty((G, mol.nao), dtype=torch.float64, device="cuda")
    args = [_dev(x) for x in (centers, l, poff, aoff, ex, co)]
    rc = L.qex_td_eval_ao(G, _lib.p(coords), len(mol.shells), *[_lib.p(a) for a in args],
                          mol.nao, _lib.p(ao), _lib.stream())
    N.check(rc, "qex_td_eval_ao")
    return ao


def eval_rho(ao, dm):
    """rho_g = sum_ij ao_gi D_ij ao_gj (LDA)."""
    torch = N.require_cuda()
    L = _lib.lib()
    ao = _dev(ao, torch.float64)
    dm = _dev(dm, torch.float64)
    G, n = ao.shape
    ws = torch.empty(max(L.qex_td_rho_workspace_size(G, n), 8), dtype=torch.uint8, device="cuda")
    rho = torch.empty(G, dtype=torch.float64, device="cuda")
    N.check(L.qex_td_rho(G, n, _lib.p(ao), _lib.p(dm), _lib.p(rho), _lib.p(ws), ws.numel(),
                         _lib.stream()), "qex_td_rho")
    return rho


def eval_xc_lda(rho, weights, vwn=False):
    """(exc, vrho, nelec, excsum) of the Slater exchange on the grid; with ``vwn``
    plus the VWN correlation (the reference's default "LDA,VWN")."""
    torch = N.require_cuda()
    L = _lib.lib()
    rho = _dev(rho, torch.float64)
    weights = _dev(weights, torch.float64)
    G = rho.shape[0]
    exc = torch.empty_like(rho)
    vrho = torch.empty_like(rho)
    sums = torch.empty(2, dtype=torch.float64, device="cuda")
    ws = torch.empty(L.qex_td_lda_workspace_size(G), dtype=torch.uint8, device="cuda")
    fn = L.qex_td_lda_vwn if vwn else L.qex_td_lda
    N.check(fn(G, _lib.p(rho), _lib.p(weights), _lib.p(exc), _lib.p(vrho), _lib.p(sums),
               _lib.p(ws), ws.numel(), _lib.stream()), "qex_td_lda")
    return exc, vrho, sums[0], sums[1]


class NeuralXC:
    """Neural XC functional of the 3D path (qedft/train/td/trainer_legacy_no_jit.py:98-107:
    MLP features [H, H, 1], gelu hidden layers, output -scale * swish).  Local form
    (Dense_0 kernel (1, H)): evaluated per grid point (:56-62), exc per point.  Global
    form (Dense_0 kernel (G, H)): the density vector is one input (:46-53), exc is the
    scalar sum of the output.  ``params`` is the flax parameter tree
    ``{"Dense_0": {"kernel": (in, H), "bias": (H,)}, "Dense_1": ..., "Dense_2": ...}`` or,
    for the local form, the flat FP32 vector (w1, b1, W2, b2, w3, b3)."""

    def __init__(self, params, scale=1e-2):
        import numpy as np

        self.scale = float(scale)
        self.inputs = 1
        if isinstance(params, dict):
            d0, d1, d2 = params["Dense_0"], params["Dense_1"], params["Dense_2"]
            flat = np.concatenate([np.ravel(d0["kernel"]), np.ravel(d0["bias"]),
                                   np.ravel(d1["kernel"]), np.ravel(d1["bias"]),
                                   np.ravel(d2["kernel"]), np.ravel(d2["bias"])])
            self.hidden = int(np.shape(d0["bias"])[0])
            self.inputs = int(np.shape(d0["kernel"])[0])
        else:
            flat = np.ravel(np.asarray(params))
            self.hidden = int(round((-3 + (9 + 4 * (flat.size - 1)) ** 0.5) / 2))
        H = self.hidden
        if flat.size != H * H + (2 + self.inputs + 1) * H + 1:
            raise ValueError(f"parameter vector of {flat.size} floats does not fit [H, H, 1]")
        self.flat = np.ascontiguousarray(flat, dtype=np.float32)
        self._dev = None

    @property
    def is_global(self):
        return self.inputs > 1

    @staticmethod
    def init(hidden=512, seed=0, inputs=1):
        """flax-style initialisation: lecun-normal kernels, zero biases; ``inputs`` =
        1 for the local form, the number of grid points for the global form."""
        import numpy as np

        rng = np.random.default_rng(seed)

        def dense(fi, fo):
            return {"kernel": rng.normal(0.0, 1.0 / np.sqrt(fi), (fi, fo)).astype(np.float32),
                    "bias": np.zeros(fo, np.float32)}

        return {"Dense_0": dense(inputs, hidden), "Dense_1": dense(hidden, hidden),
                "Dense_2": dense(hidden, 1)}

    def device_params(self):
        torch = N.require_cuda()
        if self._dev is None:
            self._dev = torch.as_tensor(self.flat, device="cuda")
        return self._dev


def eval_xc_nn(rho, functional: NeuralXC, weights=None):
    """(exc, vrho) = (network(rho), d network / d rho) per grid point, as
    ``get_exc_and_vrho`` (qedft/train/td/xc.py:12-47) returns them; with
    ``weights`` also (nelec, excsum) = (sum w rho, sum w rho exc)."""
    torch = N.require_cuda()
    L = _lib.lib()
    rho = _dev(rho, torch.float64)
    G = rho.shape[0]
    H = functional.hidden
    w = None if weights is None else _dev(weights, torch.float64)
    if functional.is_global:
        # exc is one number (the network's summed output); nr_rks adds it as excsum
        if functional.inputs != G:
            raise ValueError(f"global network over {functional.inputs} points, grid has {G}")
        if w is None:
            raise ValueError("the global network needs the grid weights")
        vrho = torch.empty_like(rho)
        sums = torch.empty(2, dtype=torch.float64, device="cuda")
        ws = torch.empty(max(L.qex_td_nn_xc_global_workspace_size(G, H), 256), dtype=torch.uint8,
                         device="cuda")
        N.check(L.qex_td_nn_xc_global(G, H, _lib.p(rho), _lib.p(w),
                                      _lib.p(functional.device_params()), functional.scale,
                                      _lib.p(vrho), _lib.p(sums), _lib.p(ws), ws.numel(),
                                      _lib.stream()), "qex_td_nn_xc_global")
        return None, vrho, sums[0], sums[1]
    exc = torch.empty_like(rho)
    vrho = torch.empty_like(rho)
    sums = None if w is None else torch.empty(2, dtype=torch.float64, device="cuda")
    ws = torch.empty(max(L.qex_td_nn_xc_workspace_size(G, H), 256), dtype=torch.uint8,
                     device="cuda")
    N.check(L.qex_td_nn_xc(G, H, _lib.p(rho), _lib.p(w), _lib.p(functional.device_params()),
                           functional.scale, _lib.p(exc), _lib.p(vrho), _lib.p(sums),
                           _lib.p(ws), ws.numel(), _lib.stream()), "qex_td_nn_xc")
    if w is None:
        return exc, vrho
    return exc, vrho, sums[0], sums[1]


def vxc_matrix(ao, weights, vrho):
    """ao^T diag(0.5 w v) ao + its transpose."""
    torch = N.require_cuda()
    L = _lib.lib()
    ao = _dev(ao, torch.float64)
    G, n = ao.shape
    vmat = torch.empty((n, n), dtype=torch.float64, device="cuda")
    ws = torch.empty(max(L.qex_td_vxc_workspace_size(G, n), 8), dtype=torch.uint8, device="cuda")
    N.check(L.qex_td_vxc(G, n, _lib.p(ao), _lib.p(_dev(weights, torch.float64)),
                         _lib.p(_dev(vrho, torch.float64)), _lib.p(vmat), _lib.p(ws), ws.numel(),
                         _lib.stream()), "qex_td_vxc")
    return vmat


GGA_CODES = ("PBE_X", "GGA_X_PBE")
_LDA_CODES = ("LDA", "LDA_X", "SLATER", "LDA,VWN", "SLATER,VWN")


def eval_ao_deriv1(mol, coords=None):
    """(4, G, nao): AO values and their x, y, z derivatives (pyscf's ao_deriv = 1
    layout, as the GGA branch of ``numint_legacy.py:175-177`` requests)."""
    torch = N.require_cuda()
    L = _lib.lib()
    coords = _dev(mol.coords if coords is None else coords, torch.float64)
    centers, l, poff, aoff, ex, co = mol.shell_arrays()
    G = coords.shape[0]
    ao4 = torch.empty((4, G, mol.nao), dtype=torch.float64, device="cuda")
    args = [_dev(x) for x in (centers, l, poff, aoff, ex, co)]
    N.check(L.qex_td_eval_ao_deriv1(G, _lib.p(coords), len(mol.shells),
                                    *[_lib.p(a) for a in args], mol.nao, _lib.p(ao4),
                                    _lib.stream()), "qex_td_eval_ao_deriv1")
    return ao4


def eval_rho_gga(ao4, dm):
    """(4, G): rho and its gradient (make_rho "GGA", ``numint_legacy.py:180,351-397``)."""
    torch = N.require_cuda()
    L = _lib.lib()
    ao4 = _dev(ao4, torch.float64)
    dm = _dev(dm, torch.float64)
    _, G, n = ao4.shape
    ws = torch.empty(max(L.qex_td_rho_gga_workspace_size(G, n), 8), dtype=torch.uint8,
                     device="cuda")
    rho4 = torch.empty((4, G), dtype=torch.float64, device="cuda")
    N.check(L.qex_td_rho_gga(G, n, _lib.p(ao4), _lib.p(dm), _lib.p(rho4), _lib.p(ws), ws.numel(),
                             _lib.stream()), "qex_td_rho_gga")
    return rho4


def eval_xc_pbe_x(rho4, weights):
    """PBE exchange on the grid: (exc, wv, nelec, excsum), wv the GGA potential
    weights of ``_rks_gga_wv0`` (0.5 w vrho, 2 w vsigma grad rho)."""
    torch = N.require_cuda()
    L = _lib.lib()
    G = rho4.shape[1]
    w = _dev(weights, torch.float64)
    exc = torch.empty(G, dtype=torch.float64, device="cuda")
    wv = torch.empty((4, G), dtype=torch.float64, device="cuda")
    sums = torch.empty(2, dtype=torch.float64, device="cuda")
    ws = torch.empty(max(L.qex_td_gga_pbe_x_workspace_size(G), 8), dtype=torch.uint8,
                     device="cuda")
    N.check(L.qex_td_gga_pbe_x(G, _lib.p(rho4), _lib.p(w), _lib.p(exc), _lib.p(wv), _lib.p(sums),
                               _lib.p(ws), ws.numel(), _lib.stream()), "qex_td_gga_pbe_x")
    return exc, wv, sums[0], sums[1]


def vxc_matrix_gga(ao4, wv):
    """ao0^T (sum_n wv_n o ao_n) + transpose (``numint_legacy.py:194-196,337``)."""
    torch = N.require_cuda()
    L = _lib.lib()
    _, G, n = ao4.shape
    ws = torch.empty(max(L.qex_td_vxc_gga_workspace_size(G, n), 8), dtype=torch.uint8,
                     device="cuda")
    vmat = torch.empty((n, n), dtype=torch.float64, device="cuda")
    N.check(L.qex_td_vxc_gga(G, n, _lib.p(ao4), _lib.p(wv), _lib.p(vmat), _lib.p(ws), ws.numel(),
                             _lib.stream()), "qex_td_vxc_gga")
    return vmat


def nr_rks_gga(ao4, weights, dm, xc_code="PBE_X"):
    """(nelec, excsum, vmat) of the GGA branch of ``numint_legacy.py:175-198``."""
    code = xc_code.upper().replace(" ", "")
    if code not in GGA_CODES:
        raise NotImplementedError(f"GGA xc_code {xc_code!r}: the GPU path implements PBE exchange")
    rho4 = eval_rho_gga(ao4, dm)
    _, wv, nelec, excsum = eval_xc_pbe_x(rho4, weights)
    return nelec, excsum, vxc_matrix_gga(ao4, wv)


def nr_rks(ao, weights, dm, xc_code="LDA"):
    """(nelec, excsum, vmat) (``numint_legacy.py:122-164,337``) for the LDA exchange,
    with a ``NeuralXC`` as ``xc_code`` the neural functional (``xc.py:57-87``),
    or a GGA code ("PBE_X") with ``ao`` the (4, G, nao) values and gradients."""
    if isinstance(xc_code, str) and xc_code.upper().replace(" ", "") in GGA_CODES:
        return nr_rks_gga(ao, weights, dm, xc_code)
    rho = eval_rho(ao, dm)
    if isinstance(xc_code, NeuralXC):
        exc, vrho, nelec, excsum = eval_xc_nn(rho, xc_code, weights)
        return nelec, excsum, vxc_matrix(ao, weights, vrho)
    code = xc_code.upper().replace(" ", "")
    if code not in _LDA_CODES:
        raise NotImplementedError(f"xc_code {xc_code!r}: the GPU path implements the LDA exchange "
                                  "(with or without VWN correlation) and the neural functional")
    exc, vrho, nelec, excsum = eval_xc_lda(rho, weights, vwn=code.endswith("VWN"))
    return nelec, excsum, vxc_matrix(ao, weights, vrho)


class NumInt:
    """The reference's ``NumInt`` interface (``qedft/train/td/numint.py:16-273``
    ``nr_rks``, and ``eval_rho`` / ``eval_xc`` of ``:276-400``) over the GPU
    kernels.

    ``mol``: a molecule with Cartesian shells (``shells``, ``nao``,
    ``shell_arrays()``, e.g. ``workloads.Molecule3D``).  ``grids``: anything
    with ``coords`` (G, 3) and ``weights`` (G,), such as
    ``qex_gb300.td.grids.Grids`` after ``build()`` or the molecule itself.
    ``xc_code``: "LDA" / "LDA_X" / "SLATER" (Slater exchange), "LDA,VWN" (the
    reference's default), "PBE_X" (GGA), or a code containing "NN" with the
    network passed as ``params`` (a ``NeuralXC`` or its flax parameter tree).
    ``dms``: one (nao, nao) density matrix or a stack of them; the results are
    per matrix, unwrapped for a single one, as the reference returns them.
    ``relativity``, ``hermi``, ``max_memory`` and ``verbose`` are accepted for
    the reference's signature; the GPU path holds the whole grid at once.
    """

    @staticmethod
    def _functional(xc_code, params):
        if isinstance(xc_code, NeuralXC):
            return xc_code
        if isinstance(xc_code, str) and "NN" in xc_code.upper():
            if params is None:
                raise ValueError(f"xc_code {xc_code!r} needs the network as params")
            return params if isinstance(params, NeuralXC) else NeuralXC(params)
        return xc_code

    @staticmethod
    def _code(xc):
        return xc.upper().replace(" ", "") if isinstance(xc, str) else None

    def nr_rks(self, mol, grids, xc_code, dms, relativity=0, hermi=0, max_memory=2000,
               verbose=None, params=None):
        torch = N.require_cuda()
        xc = self._functional(xc_code, params)
        gga = self._code(xc) in GGA_CODES
        ao = eval_ao_deriv1(mol, grids.coords) if gga else eval_ao(mol, grids.coords)
        d = _dev(dms, torch.float64)
        single = d.dim() == 2
        parts = [nr_rks(ao, grids.weights, dm, xc) for dm in (d[None] if single else d)]
        nelec, excsum, vmat = ([p[k] for p in parts] for k in range(3))
        if single:
            return nelec[0], excsum[0], vmat[0]
        return nelec, excsum, vmat

    def eval_rho(self, mol, ao, dm, non0tab=None, xctype="LDA", hermi=0, verbose=None):
        """rho (LDA, from (G, nao) AO values) or rho and its gradient (GGA, from
        the (4, G, nao) values and derivatives)."""
        kind = xctype.upper()
        if kind == "LDA":
            return eval_rho(ao, dm)
        if kind == "GGA":
            return eval_rho_gga(ao, dm)
        raise NotImplementedError(f"xctype {xctype!r}: the GPU path evaluates LDA and GGA densities")

    @staticmethod
    def eval_xc(xc_code, rho, spin=0, relativity=0, deriv=1, verbose=None, params=None,
                weights=None):
        """(exc, (vrho, None, None, None), None, None) of an LDA or neural
        functional (``qedft/train/td/xc.py:57-87``); ValueError unless deriv == 1,
        as the reference.  The global neural form needs the grid ``weights``."""
        if deriv != 1:
            raise ValueError("eval_xc: deriv should be set to 1.")
        if spin != 0:
            raise NotImplementedError("spin-polarised functionals are not on the GPU path")
        xc = NumInt._functional(xc_code, params)
        if isinstance(xc, NeuralXC):
            if xc.is_global:
                raise NotImplementedError("the global network's exc is one number: use nr_rks")
            exc, vrho = eval_xc_nn(rho, xc)
        elif NumInt._code(xc) in _LDA_CODES:
            torch = N.require_cuda()
            r = _dev(rho, torch.float64)
            w = torch.ones_like(r) if weights is None else weights
            exc, vrho, _, _ = eval_xc_lda(r, w, vwn=NumInt._code(xc).endswith("VWN"))
        else:
            raise NotImplementedError(f"eval_xc for {xc_code!r}: LDA and neural functionals "
                                      "(GGA through nr_rks)")
        return exc, (vrho, None, None, None), None, None
