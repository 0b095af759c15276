"""DMFT drivers on top of the GPU impurity solver (cmpy/dmft/twosite.py, cmpy/dmft/utils.py).

Two parts:

* the reference's two-site DMFT at half filling (cmpy/dmft/twosite.py:103-172) with its
  helpers (self energy, Bethe-lattice Green's function, quasiparticle weight, mixing,
  iteration statistics; cmpy/dmft/utils.py:66-260) and the analytic two-site solution of
  E. Lange (twosite.py:25-84). The impurity Green's function comes from the engine
  (`SingleImpurityAndersonModel.impurity_gf`, thermal Lehmann sum on the device) or, at
  T = 0, from the ground state and the zero-temperature Lehmann sum;
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
# helpers (cmpy/dmft/utils.py)
# ------------------------------------------------------------------------------------------


class IterationStats(Sequence):
    """Errors per iteration and the convergence status (cmpy/dmft/utils.py:66-160)."""

    def __init__(self, *labels):
        super().__init__()
        self._errors = []
        self.labels = labels
        self.success = False
        self.status = ""

    @property
    def iteration(self):
        return len(self._errors)

    @property
    def errors(self):
        return self._errors[-1]

    @property
    def history(self):
        return np.asarray(self._errors).T

    @property
    def message(self):
        msg = "Self-consistency reached" if self.success else "Self-consistency not reached"
        return msg + ": " + self.status

    def append(self, *items):
        self._errors.append(list(items))

    def set_status(self, success, status=""):
        self.success = success
        self.status = status

    def set_maxiter_status(self, maxiter):
        self.success = False
        self.status = f"Maximum iteration of {maxiter} reached without converging!"

    def set_parameter_converged(self, name, value, dec=4):
        self.success = True
        self.status = f"{name} converged to {value:.{dec}f}"

    def __bool__(self):
        return self.success

    def __len__(self):
        return len(self._errors)

    def __getitem__(self, i):
        return self._errors[i]

    def __str__(self):
        return f"{self.message} (iterations: {self.iteration})"


def mix_values(old, new, mixing=1.0):
    """new * mixing + old * (1 - mixing); mixing = 1 returns `new` (cmpy/dmft/utils.py:163-185)."""
    if mixing == 1:
        return new
    assert 0 < mixing < 1
    return new * mixing + old * (1.0 - mixing)


def self_energy(gf_imp0, gf_imp):
    """Sigma(z) = G0(z)^-1 - G(z)^-1 (cmpy/dmft/utils.py:188-211)."""
    return 1 / gf_imp0 - 1 / gf_imp


def bethe_gf_omega(z, t: float):
    """Local Green's function of the Bethe lattice (infinite coordination, hopping t)
    (cmpy/dmft/utils.py:214-230)."""
    z_rel = z / (2 * t)
    return z_rel * (1 - np.sqrt(1 - 1 / (z_rel * z_rel))) / t


def quasiparticle_weight(omegas, sigma, thresh: float = 1e-5):
    """z_qp = [1 - dRe Sigma/domega (0)]^-1 from a linear fit over the frequencies within one
    grid step of 0; set to 0 below `thresh` (cmpy/dmft/utils.py:233-275)."""
    omegas = np.asarray(omegas)
    sigma = np.asarray(sigma)
    dw = omegas[1] - omegas[0]
    win = (-dw <= omegas) * (omegas <= +dw)
    try:
        dsigma = np.polyfit(omegas[win], sigma.real[win], 1)[0]
    except np.linalg.LinAlgError:
        omega_win = omegas[win]
        sigma_win = sigma[win]
        dsigma = (sigma_win[-1] - sigma_win[0]) / (omega_win[-1] - omega_win[0])
    z_qp = 1 / (1 - dsigma)
    if z_qp < thresh:
        z_qp = 0
    return z_qp


# ------------------------------------------------------------------------------------------
# two-site DMFT (cmpy/dmft/twosite.py)
# ------------------------------------------------------------------------------------------


def impurity_params_ref(u: float, v: float):
    """Residues and poles of the two-site SIAM Green's function at half filling and T = 0
    (E. Lange; cmpy/dmft/twosite.py:25-60): (alpha_1, alpha_2, omega_1, omega_2)."""
    sqrt16 = np.sqrt(u**2 + 16 * v**2)
    sqrt64 = np.sqrt(u**2 + 64 * v**2)
    a1 = 0.25 * (1 - (u**2 - 32 * v**2) / np.sqrt((u**2 + 64 * v**2) * (u**2 + 16 * v**2)))
    a2 = 0.5 - a1
    e1 = 0.25 * (sqrt64 - sqrt16)
    e2 = 0.25 * (sqrt64 + sqrt16)
    return float(a1), float(a2), float(e1), float(e2)


def impurity_gf_ref(z, u: float, v: float):
    """Analytic two-site impurity Green's function (cmpy/dmft/twosite.py:63-84)."""
    a1, a2, e1, e2 = impurity_params_ref(u, v)
    return (a1 / (z - e1) + a1 / (z + e1)) + (a2 / (z - e2) + a2 / (z + e2))


def impurity_gf0(z, siam):
    return siam.impurity_gf0(z)


def _impurity_gf_t0(z, siam: SingleImpurityAndersonModel):
    """T = 0 impurity Green's function from the ground state (the reference's thermal path
    divides by temp = 0 here)."""
    from .exactdiag import compute_groundstate, gf_lehmann_zero_temperature

    gs = compute_groundstate(siam)
    return gf_lehmann_zero_temperature(siam, z, gs.energy, gs.state, gs.n_up, gs.n_dn, pos=0)


def compute_impurity_gf(z, siam, ref=False):
    """Impurity Green's function: Lange's analytic two-site result (ref=True) or the engine
    (thermal Lehmann sum on the device; ground state + T = 0 Lehmann sum when temp = 0)."""
    if ref:
        return impurity_gf_ref(z, float(np.atleast_1d(siam.u)[0]), float(siam.v[0]))
    if siam.temp == 0:
        return _impurity_gf_t0(z, siam)
    return siam.impurity_gf(z)


def compute_self_energy(z, siam, ref=False):
    gf_imp0 = impurity_gf0(z, siam)
    gf_imp = compute_impurity_gf(z, siam, ref=ref)
    return self_energy(gf_imp0, gf_imp)


def twosite_dmft_half_filling(z, u, t=1.0, beta=np.inf, mixing=1.0, vtol=1e-6, max_iter=1000, vthresh=1e-10,
                              verbose=True, ref=True):
    """Two-site DMFT of the half-filled Hubbard model on the Bethe lattice (M. Potthoff's
    scheme, cmpy/dmft/twosite.py:103-172): the bath hybridisation is updated to
    v = sqrt(z_qp * m2) with m2 = t^2 until it changes by less than vtol. Returns the SIAM
    (its ``stats`` attribute holds the iteration history)."""
    siam = SingleImpurityAndersonModel(u, v=[t], mu=u / 2, temp=0.0 if not np.isfinite(beta) else 1 / beta)
    v = siam.v[0] + 0.1  # the first update must differ from the initial value
    m2 = t**2
    it = 0
    stats = IterationStats("Δv")
    while True:
        siam.update_hybridization(v)
        gf_imp0 = impurity_gf0(z, siam)
        gf_imp = compute_impurity_gf(z, siam, ref=ref)
        sigma = self_energy(gf_imp0, gf_imp)
        qp_weight = quasiparticle_weight(z.real, sigma, thresh=vthresh)
        v_new = mix_values(v, np.sqrt(qp_weight * m2), mixing=mixing)
        delta_v = np.linalg.norm(v - v_new)
        stats.append(delta_v)
        v = v_new
        if v == 0:
            stats.set_parameter_converged("Hybridization", v)
            break
        if delta_v < vtol:
            stats.set_parameter_converged("Hybridization", v)
            break
        elif qp_weight == 0:
            stats.set_parameter_converged("Quasiparticle weight", qp_weight)
            break
        elif it >= max_iter:
            stats.set_maxiter_status(max_iter)
            break
        it += 1
    siam.update_hybridization(v)
    object.__setattr__(siam, "stats", stats)
    if verbose:
        print("-" * 50)
        print(f"U:          {u:.2f}")
        print(stats)
    return siam


def compute_lattice_greens_function(z, siam, t, ref=False):
    """G_latt(z) = G_Bethe(z + mu - Sigma(z)) (cmpy/dmft/twosite.py:175-178)."""
    mu = siam.mu
    sigma = compute_self_energy(z, siam, ref)
    return bethe_gf_omega(z + mu - sigma, t)


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
