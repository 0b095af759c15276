"""DMFT drivers on top of the GPU impurity solver (cmpy/dmft/twosite.py, cmpy/dmft/utils.py).

Two parts:

* two-site DMFT at half filling (the entry point of cmpy/dmft/twosite.py:103-172, written
  here from the physics: V^2 = Z t^2 on the Bethe lattice) with the public helpers of
  cmpy/dmft/utils.py (self energy, Bethe-lattice Green's function, quasiparticle weight,
  mixing, iteration record) and E. Lange's closed-form two-site solution. The impurity
  Green's function comes from the engine (`SingleImpurityAndersonModel.impurity_gf`, thermal
  Lehmann sum on the device) or, at T = 0, from the ground state and the zero-temperature
  Lehmann sum;
* a multi-bath DMFT loop on the Matsubara axis for the Bethe lattice with a bath fit that
  uses the adjoint Green's function (`cmpy_gb300.adjoint`): the bath energies and
  hybridisations are fitted so that the impurity Green's function of the SIAM matches a
  target, with gradients from reverse-mode Lanczos (the reference only updates bath
  parameters by hand, cmpy/models/anderson.py:93-125).

Plotting helpers of the reference (matplotlib) are not part of this module.
"""

from __future__ import annotations

from collections.abc import Sequence
from dataclasses import dataclass, field

import numpy as np
import torch

from .models import SingleImpurityAndersonModel

__all__ = [
    "IterationStats",
    "mix_values",
    "self_energy",
    "bethe_gf_omega",
    "quasiparticle_weight",
    "impurity_params_ref",
    "impurity_gf_ref",
    "impurity_gf0",
    "compute_impurity_gf",
    "compute_self_energy",
    "twosite_dmft_half_filling",
    "compute_lattice_greens_function",
    "fit_hybridization",
    "fit_impurity_gf",
    "DMFTResult",
    "dmft_bethe_matsubara",
]


# ------------------------------------------------------------------------------------------
# loop bookkeeping and the Green's-function algebra of the DMFT cycle
# (public names as cmpy/dmft/utils.py:66-275)
# ------------------------------------------------------------------------------------------


class IterationStats(Sequence):
    """Record of a self-consistency loop: one row of monitored quantities (``labels``) per
    iteration, and the outcome once the loop has ended (``success``, ``status``)."""

    def __init__(self, *labels):
        self.labels = tuple(labels)
        self._rows: list = []
        self.success = False
        self.status = ""

    # the rows
    def append(self, *values):
        self._rows.append([float(np.real(v)) for v in values])

    def __len__(self):
        return len(self._rows)

    def __getitem__(self, i):
        return self._rows[i]

    @property
    def iteration(self):
        return len(self._rows)

    @property
    def errors(self):
        """The monitored quantities of the latest iteration."""
        return self._rows[-1]

    @property
    def history(self):
        """Array [len(labels), iterations]."""
        return np.array(self._rows, dtype=np.float64).T

    # the outcome
    def set_status(self, success, status=""):
        self.success, self.status = bool(success), str(status)

    def set_maxiter_status(self, maxiter):
        self.set_status(False, f"stopped after {maxiter} iterations")

    def set_parameter_converged(self, name, value, dec=4):
        self.set_status(True, f"{name} settled at {value:.{dec}f}")

    @property
    def message(self):
        return ("converged" if self.success else "not converged") + (f" ({self.status})" if self.status else "")

    def __bool__(self):
        return self.success

    def __str__(self):
        return f"{self.message} after {self.iteration} iterations"


def mix_values(old, new, mixing=1.0):
    """Linear mixing old + mixing * (new - old); mixing must lie in (0, 1]."""
    if not 0 < mixing <= 1:
        raise ValueError("mixing must lie in (0, 1]")
    return new if mixing == 1 else old + mixing * (new - old)


def self_energy(gf_imp0, gf_imp):
    """Dyson equation: Sigma(z) = G0(z)^-1 - G(z)^-1."""
    return 1.0 / gf_imp0 - 1.0 / gf_imp


def bethe_gf_omega(z, t: float):
    """Local Green's function of the Bethe lattice with hopping t (semicircular density of
    states of half-width 2t): G(z) = 2 / (z (1 + sqrt(1 - 4 t^2 / z^2))), the form that is
    stable for large |z| and has Im G < 0 for Im z > 0."""
    z = np.asarray(z, dtype=np.complex128)
    return 2.0 / (z * (1.0 + np.sqrt(1.0 - 4.0 * t * t / (z * z))))


def quasiparticle_weight(omegas, sigma, thresh: float = 1e-5):
    """Z = 1 / (1 - d Re Sigma / d omega) at omega = 0, the slope taken as the central
    difference of Re Sigma interpolated one grid step on either side of 0; Z below `thresh`
    counts as 0 (an insulator)."""
    w = np.asarray(omegas, dtype=np.float64)
    s = np.asarray(sigma).real
    h = abs(w[1] - w[0])
    slope = (np.interp(h, w, s) - np.interp(-h, w, s)) / (2.0 * h)
    z_qp = 1.0 / (1.0 - slope)
    return 0 if z_qp < thresh else z_qp


# ------------------------------------------------------------------------------------------
# two-site DMFT (the scheme of M. Potthoff; reference driver cmpy/dmft/twosite.py:103-172)
# ------------------------------------------------------------------------------------------


def impurity_params_ref(u: float, v: float):
    """Closed-form Green's function of the half-filled two-site Anderson impurity at T = 0
    (E. Lange): four poles at +-omega_1, +-omega_2 with weights alpha_1, alpha_2,
    omega_{1,2} = (sqrt(U^2 + 64 V^2) -+ sqrt(U^2 + 16 V^2)) / 4,
    alpha_1 = (1 - (U^2 - 32 V^2) / sqrt((U^2 + 64 V^2)(U^2 + 16 V^2))) / 4, alpha_2 = 1/2 - alpha_1.
    Returns (alpha_1, alpha_2, omega_1, omega_2)."""
    r64, r16 = np.sqrt(u * u + 64.0 * v * v), np.sqrt(u * u + 16.0 * v * v)
    alpha1 = 0.25 - 0.25 * (u * u - 32.0 * v * v) / (r64 * r16)
    return float(alpha1), float(0.5 - alpha1), float(0.25 * (r64 - r16)), float(0.25 * (r64 + r16))


def impurity_gf_ref(z, u: float, v: float):
    """Lange's two-site impurity Green's function, each +-omega pole pair combined:
    sum_k alpha_k 2 z / (z^2 - omega_k^2)."""
    a1, a2, w1, w2 = impurity_params_ref(u, v)
    z = np.asarray(z, dtype=np.complex128)
    return 2.0 * z * (a1 / (z * z - w1 * w1) + a2 / (z * z - w2 * w2))


def impurity_gf0(z, siam):
    return siam.impurity_gf0(z)


def _impurity_gf_t0(z, siam: SingleImpurityAndersonModel):
    """T = 0 impurity Green's function from the ground state (the reference's thermal path
    divides by temp = 0 here)."""
    from .exactdiag import compute_groundstate, gf_lehmann_zero_temperature

    gs = compute_groundstate(siam)
    return gf_lehmann_zero_temperature(siam, z, gs.energy, gs.state, gs.n_up, gs.n_dn, pos=0)


def compute_impurity_gf(z, siam, ref=False):
    """Impurity Green's function: Lange's closed form (ref=True) or the engine (thermal
    Lehmann sum on the device; ground state + T = 0 Lehmann sum when temp = 0)."""
    if ref:
        return impurity_gf_ref(z, float(np.atleast_1d(siam.u)[0]), float(siam.v[0]))
    return _impurity_gf_t0(z, siam) if siam.temp == 0 else siam.impurity_gf(z)


def compute_self_energy(z, siam, ref=False):
    return self_energy(impurity_gf0(z, siam), compute_impurity_gf(z, siam, ref=ref))


def twosite_dmft_half_filling(z, u, t=1.0, beta=np.inf, mixing=1.0, vtol=1e-6, max_iter=1000, vthresh=1e-10,
                              verbose=True, ref=True):
    """Two-site DMFT of the half-filled Hubbard model on the Bethe lattice. The bath of the
    one-bath-site impurity is fixed by matching the low-frequency weight of the lattice: the
    hybridisation obeys V^2 = Z t^2 with Z the quasiparticle weight of the impurity self
    energy. Starting from the free value V = t, the map V -> sqrt(Z(V)) t is iterated (with
    linear mixing) until V moves by less than `vtol`, Z vanishes (Mott insulator) or
    `max_iter` is reached. Returns the SIAM at the fixed point; its ``stats`` attribute holds
    the history of |dV|."""
    temp = 1.0 / beta if np.isfinite(beta) else 0.0
    siam = SingleImpurityAndersonModel(u, v=[t], mu=u / 2, temp=temp)
    stats = IterationStats("dv")
    omegas = np.asarray(z).real
    v = float(t)
    for _ in range(max_iter + 1):
        siam.update_hybridization(v)
        z_qp = quasiparticle_weight(omegas, compute_self_energy(z, siam, ref=ref), thresh=vthresh)
        v_next = float(mix_values(v, t * np.sqrt(z_qp), mixing=mixing))
        stats.append(abs(v_next - v))
        v = v_next
        if z_qp == 0 or v == 0:
            stats.set_parameter_converged("quasiparticle weight", 0.0)
            break
        if stats.errors[0] < vtol:
            stats.set_parameter_converged("hybridisation", v)
            break
    else:
        stats.set_maxiter_status(max_iter)
    siam.update_hybridization(v)
    object.__setattr__(siam, "stats", stats)
    if verbose:
        print(f"two-site DMFT, U = {u:g}: V = {v:.8f}, {stats}")
    return siam


def compute_lattice_greens_function(z, siam, t, ref=False):
    """Local lattice Green's function G_Bethe(z + mu - Sigma(z))."""
    return bethe_gf_omega(z + siam.mu - compute_self_energy(z, siam, ref), t)


# ------------------------------------------------------------------------------------------
# multi-bath DMFT on the Matsubara axis with adjoint bath fits (no reference counterpart)
# ------------------------------------------------------------------------------------------


def _bath_theta(eps_bath: torch.Tensor, v: torch.Tensor, u: float, mu: float):
    """theta of the SIAM with the physical fermionic hopping signs (sign width = number of
    sites; the reference's SIAM passes width 0, cmpy/models/anderson.py:149, which changes the
    spectrum as soon as a bond passes over occupied bath sites)."""
    from .adjoint import siam_parameters

    dev = eps_bath.device
    theta, ns, bonds, _ = siam_parameters(torch.tensor(float(u), dtype=torch.float64, device=dev),
                                          torch.tensor(0.0, dtype=torch.float64, device=dev), eps_bath, v,
                                          mu=torch.tensor(float(mu), dtype=torch.float64, device=dev))
    return theta, ns, bonds, ns


def fit_hybridization(iwn, delta_target, eps_bath0, v0, steps: int = 400, lr: float = 0.05):
    """Bath (eps_k, V_k) minimising sum_n |Delta(i w_n) - Delta_target|^2 with
    Delta(z) = sum_k V_k^2/(z - eps_k) (cmpy/models/anderson.py:127-145); torch autograd,
    L-BFGS. Returns (eps_bath, v) as numpy arrays and the final loss."""
    dev = torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")
    z = torch.as_tensor(np.asarray(iwn), dtype=torch.complex128, device=dev)
    target = torch.as_tensor(np.asarray(delta_target), dtype=torch.complex128, device=dev)
    eb = torch.tensor(np.asarray(eps_bath0, dtype=np.float64), device=dev, requires_grad=True)
    vv = torch.tensor(np.asarray(v0, dtype=np.float64), device=dev, requires_grad=True)
    opt = torch.optim.LBFGS([eb, vv], lr=lr, max_iter=steps, tolerance_grad=1e-14, tolerance_change=1e-16,
                            history_size=50, line_search_fn="strong_wolfe")

    def closure():
        opt.zero_grad()
        d = torch.sum(vv**2 / (z[:, None] - eb[None, :]), dim=1)
        loss = torch.sum(torch.abs(d - target) ** 2)
        loss.backward()
        return loss

    opt.step(closure)
    with torch.no_grad():  # LBFGS.step returns the loss of its first evaluation
        d = torch.sum(vv**2 / (z[:, None] - eb[None, :]), dim=1)
        loss = float(torch.sum(torch.abs(d - target) ** 2))
    return eb.detach().cpu().numpy(), np.abs(vv.detach().cpu().numpy()), loss


def fit_impurity_gf(iwn, g_target, u: float, eps_bath0, v0, mu: float | None = None, steps: int = 30,
                    gs_steps: int = 200, gf_levels: int = 120, ckpt: int = 16, lr: float = 1.0):
    """Bath (eps_k, V_k) of a SIAM whose interacting impurity Green's function matches g_target
    on the Matsubara frequencies: minimise sum_n |G_imp(i w_n) - g_target|^2 with gradients from
    the adjoint Green's function (reverse-mode Lanczos). The sector is half filling of the
    1 + N_b sites (N_b odd gives an even site count and a spin-singlet sector). Returns
    (eps_bath, v, loss history)."""
    from .adjoint import greens_function_ad

    dev = torch.device("cuda")
    mu = u / 2 if mu is None else mu
    z = np.asarray(iwn)
    target = torch.as_tensor(np.asarray(g_target), dtype=torch.complex128, device=dev)
    eb = torch.tensor(np.asarray(eps_bath0, dtype=np.float64), device=dev, requires_grad=True)
    vv = torch.tensor(np.asarray(v0, dtype=np.float64), device=dev, requires_grad=True)
    n_sites = len(eps_bath0) + 1
    nh = n_sites // 2
    sector = (nh, n_sites - nh) if n_sites % 2 else (nh, nh)
    opt = torch.optim.LBFGS([eb, vv], lr=lr, max_iter=steps, tolerance_grad=1e-12, tolerance_change=1e-14,
                            history_size=20, line_search_fn="strong_wolfe")
    history = []

    def closure():
        opt.zero_grad()
        theta, ns, bonds, width = _bath_theta(eb, vv, u, mu)
        g = greens_function_ad(theta, ns, bonds, sector, z, sign_width=width, gs_steps=gs_steps,
                               gf_levels=gf_levels, ckpt=ckpt)
        loss = torch.sum(torch.abs(g - target) ** 2)
        loss.backward()
        history.append(float(loss.detach()))
        return loss

    opt.step(closure)
    return eb.detach().cpu().numpy(), np.abs(vv.detach().cpu().numpy()), history


@dataclass
class DMFTResult:
    eps_bath: np.ndarray
    v: np.ndarray
    g_imp: np.ndarray
    sigma: np.ndarray
    g_loc: np.ndarray
    stats: IterationStats = field(default_factory=lambda: IterationStats("Δ"))


def dmft_bethe_matsubara(u: float, t: float = 1.0, num_bath: int = 5, beta: float = 50.0, n_mats: int = 256,
                         max_iter: int = 30, tol: float = 1e-6, mixing: float = 1.0, gf_levels: int = 200,
                         seed: int = 0) -> DMFTResult:
    """Exact-diagonalisation DMFT of the half-filled Hubbard model on the Bethe lattice at
    T = 0, on the Matsubara frequencies of a fictitious inverse temperature `beta`:
      1. Delta_target(i w_n) = t^2 G_loc(i w_n) (Bethe self-consistency);
      2. fit the bath of the SIAM to Delta_target (fit_hybridization);
      3. G_imp(i w_n) from the ground state and the continued fractions on the device;
      4. Sigma = G0^-1 - G_imp^-1, G_loc = G_Bethe(i w_n + mu - Sigma).
    Stops when max |G_loc change| < tol. num_bath should be odd (an even number of sites, so
    the half-filled ground state is a spin singlet in sector (N/2, N/2)). The SIAM uses the
    physical fermionic hopping signs (the reference's width-0 quirk makes a star with several
    bath sites a different Hamiltonian, and the loop then does not converge)."""
    from .exactdiag import compute_groundstate, gf_continued_fraction

    rng = np.random.default_rng(seed)
    iwn = 1j * (2 * np.arange(n_mats) + 1) * np.pi / beta
    mu = u / 2
    g_loc = bethe_gf_omega(iwn, t)
    eb = np.sort(rng.uniform(-2 * t, 2 * t, num_bath))
    eb = eb - eb.mean()
    vv = np.full(num_bath, t / np.sqrt(num_bath))
    stats = IterationStats("Δ")
    g_imp = sigma = None
    for it in range(max_iter):
        eb, vv, _ = fit_hybridization(iwn, t * t * g_loc, eb, vv)
        siam = SingleImpurityAndersonModel(u, eps_imp=0.0, eps_bath=eb, v=vv, mu=mu, physical_signs=True)
        gs = compute_groundstate(siam)
        g_imp = gf_continued_fraction(siam, iwn, gs.n_up, gs.n_dn, gs.energy, gs.state, pos=0, n_lev=gf_levels)
        sigma = self_energy(siam.impurity_gf0(iwn), g_imp)
        g_new = mix_values(g_loc, bethe_gf_omega(iwn + mu - sigma, t), mixing=mixing)
        err = float(np.max(np.abs(g_new - g_loc)))
        stats.append(err)
        g_loc = g_new
        if err < tol:
            stats.set_parameter_converged("Local Green's function change", err, dec=8)
            break
    else:
        stats.set_maxiter_status(max_iter)
    return DMFTResult(eb, vv, g_imp, sigma, g_loc, stats)
