"""CPU restatement of the reference's exact-diagonalisation hot path (numpy / scipy).

TEST INFRASTRUCTURE ONLY — the checker for cmpy_gb300, never part of the product path.
Each function restates the reference arithmetic in vectorised numpy, keeping the
reference's operation order where results must be bit-exact (triplets, triplet matvec),
and cites the file:line it follows (paths inside the cmpy checkout). It is pinned against
golden vectors produced by the unmodified reference (tests/golden/make_golden.py).
"""

from __future__ import annotations

import numpy as np
import scipy.linalg as la
import scipy.sparse as sp

UP, DN = 1, 2


# ---- basis: cmpy/basis.py ------------------------------------------------------------------


def popcount(a: np.ndarray) -> np.ndarray:
    a = np.asarray(a, dtype=np.uint64)
    c = np.zeros(a.shape, dtype=np.int64)
    x = a.copy()
    while np.any(x):
        c += (x & np.uint64(1)).astype(np.int64)
        x >>= np.uint64(1)
    return c


def sector_states(n_sites: int, n=None) -> np.ndarray:
    """Ascending states with popcount n; all 2^N when n is None (cmpy/basis.py:644-676)."""
    allst = np.arange(2**n_sites, dtype=np.int64)
    if n is None:
        return allst
    return allst[popcount(allst) == n]


def colex_rank(states: np.ndarray) -> np.ndarray:
    """Index of each state in its popcount sector, sum_k C(p_k, k) (equals bisect_left
    into the sorted sector list, cmpy/operators.py:276-299)."""
    from math import comb

    states = np.asarray(states, dtype=np.int64)
    out = np.zeros(states.shape, dtype=np.int64)
    k = np.zeros(states.shape, dtype=np.int64)
    for p in range(63):
        bit = (states >> p) & 1
        k = k + bit
        c = np.array([comb(p, int(kk)) if kk > 0 else 0 for kk in range(64)], dtype=np.int64)
        out += np.where(bit == 1, c[k], 0)
    return out


# ---- projectors: cmpy/operators.py ----------------------------------------------------------


def weighted_element(states, values) -> np.ndarray:
    """Sequential ascending-site sum of values[i] over set bits (cmpy/operators.py:226-250)."""
    states = np.asarray(states, dtype=np.int64)
    values = np.asarray(values, dtype=np.float64)
    v = np.zeros(states.shape, dtype=np.float64)
    for i in range(values.shape[0]):
        v = np.where((states >> i) & 1 == 1, v + values[i], v)
    return v


def hop_sign(states, width: int, site1: int, site2: int) -> np.ndarray:
    """(-1)^(set bits strictly between site1 and site2 below `width`)
    (_hopping_sign + bit_count, cmpy/operators.py:253-273,425-433)."""
    states = np.asarray(states, dtype=np.int64)
    cnt = np.zeros(states.shape, dtype=np.int64)
    for i in range(site1 + 1, site2):
        if i < width:
            cnt += (states >> i) & 1
    return np.where(cnt % 2 == 1, -1, 1)


def _truthy(e):
    return (e != 0.0) | np.isnan(e)


def coo_onsite(up_states, dn_states, eps):
    """project_onsite_energy (cmpy/operators.py:359-422)."""
    up = np.asarray(up_states, dtype=np.int64)
    dn = np.asarray(dn_states, dtype=np.int64)
    nu, nd = len(up), len(dn)
    rows, vals = [], []
    e_up = weighted_element(up, eps)
    for i in np.nonzero(_truthy(e_up))[0]:
        rows.append(i * nd + np.arange(nd, dtype=np.int64))
        vals.append(np.full(nd, e_up[i]))
    e_dn = weighted_element(dn, eps)
    for j in np.nonzero(_truthy(e_dn))[0]:
        rows.append(np.arange(nu, dtype=np.int64) * nd + j)
        vals.append(np.full(nu, e_dn[j]))
    r = np.concatenate(rows) if rows else np.zeros(0, np.int64)
    v = np.concatenate(vals) if vals else np.zeros(0, np.float64)
    return r, r.copy(), v


def coo_inter(up_states, dn_states, u):
    """project_hubbard_inter (cmpy/operators.py:305-356)."""
    up = np.asarray(up_states, dtype=np.int64)
    dn = np.asarray(dn_states, dtype=np.int64)
    both = (up[:, None] & dn[None, :]).reshape(-1)
    e = weighted_element(both, u)
    idx = np.nonzero(_truthy(e))[0].astype(np.int64)
    return idx, idx.copy(), e[idx]


def coo_hopping(up_states, dn_states, num_sites, site1, site2, hop):
    """project_hopping (cmpy/operators.py:463-527) via _compute_hopping_term (:436-460)."""
    assert site1 < site2
    up = np.asarray(up_states, dtype=np.int64)
    dn = np.asarray(dn_states, dtype=np.int64)
    nu, nd = len(up), len(dn)
    rows, cols, vals = [], [], []

    def term(states):
        occ1 = (states >> site1) & 1
        occ2 = (states >> site2) & 1
        sel = np.nonzero(occ1 != occ2)[0]
        new = states[sel] ^ (1 << site1) ^ (1 << site2)
        j = np.searchsorted(states, new, side="left")
        sg = hop_sign(states[sel], num_sites, site1, site2)
        val = np.where(sg < 0, -np.float64(hop), np.float64(hop))
        return sel, j, val

    for o, t, a in zip(*term(up)):
        rows.append(o * nd + np.arange(nd))
        cols.append(t * nd + np.arange(nd))
        vals.append(np.full(nd, a))
    for o, t, a in zip(*term(dn)):
        rows.append(np.arange(nu) * nd + o)
        cols.append(np.arange(nu) * nd + t)
        vals.append(np.full(nu, a))
    cat = lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt)
    return cat(rows, np.int64), cat(cols, np.int64), cat(vals, np.float64)


def _concat(parts):
    return tuple(np.concatenate([p[k] for p in parts]) for k in range(3))


def coo_fermion(up_states, dn_states, eps, u, bonds, width):
    """Onsite, interaction, then each bond's hopping — the order of hubbard._ham_data
    (cmpy/models/hubbard.py:13-22) and SIAM._hamiltonian_data (anderson.py:147-158)."""
    parts = [coo_onsite(up_states, dn_states, eps), coo_inter(up_states, dn_states, u)]
    for i, j, t in bonds:
        parts.append(coo_hopping(up_states, dn_states, width, i, j, t))
    return _concat(parts)


def coo_fermion_rows(up_states, dn_states, eps, u, bonds, width, up_rows: int):
    """The triplets of coo_fermion whose origin lies in the first `up_rows` up-rows, in the
    same order: a bounded sample of the reference path for CPU timing."""
    up = np.asarray(up_states, dtype=np.int64)
    dn = np.asarray(dn_states, dtype=np.int64)
    nd = len(dn)
    k = int(up_rows)
    ar_k = np.arange(k, dtype=np.int64)
    ar_d = np.arange(nd, dtype=np.int64)
    rows, cols, vals = [], [], []

    def add(r, c, v):
        rows.append(r)
        cols.append(c)
        vals.append(v)

    e_up = weighted_element(up[:k], eps)
    for i in np.nonzero(_truthy(e_up))[0]:
        add(i * nd + ar_d, i * nd + ar_d, np.full(nd, e_up[i]))
    e_dn = weighted_element(dn, eps)
    for j in np.nonzero(_truthy(e_dn))[0]:
        add(ar_k * nd + j, ar_k * nd + j, np.full(k, e_dn[j]))
    e = weighted_element((up[:k, None] & dn[None, :]).reshape(-1), u)
    idx = np.nonzero(_truthy(e))[0].astype(np.int64)
    add(idx, idx, e[idx])
    for s1, s2, hop in bonds:
        for states, is_dn in ((up, False), (dn, True)):
            occ1 = (states >> s1) & 1
            occ2 = (states >> s2) & 1
            sel = np.nonzero(occ1 != occ2)[0]
            new = states[sel] ^ (1 << s1) ^ (1 << s2)
            tgt = np.searchsorted(states, new, side="left")
            sg = hop_sign(states[sel], width, s1, s2)
            val = np.where(sg < 0, -np.float64(hop), np.float64(hop))
            for o, t, a in zip(sel, tgt, val):
                if not is_dn:
                    if o < k:
                        add(o * nd + ar_d, t * nd + ar_d, np.full(nd, a))
                else:
                    add(ar_k * nd + o, ar_k * nd + t, np.full(k, a))
    return (np.concatenate(rows).astype(np.int64), np.concatenate(cols).astype(np.int64),
            np.concatenate(vals).astype(np.float64))


def hubbard_descriptor(num_sites, neighbors, inter=0.0, eps=0.0, hop=1.0, mu=0.0):
    """HubbardModel parameters as (eps[N], u[N], bonds, width) (cmpy/models/hubbard.py:13-22,75-81)."""
    energy = np.full(num_sites, eps - mu, dtype=np.float64)
    interaction = np.full(num_sites, inter, dtype=np.float64)
    bonds = [(int(i), int(j), float(hop)) for i, j in neighbors if i < j]
    return energy, interaction, bonds, num_sites


def siam_descriptor(u, eps_imp, eps_bath, v, mu=None):
    """SingleImpurityAndersonModel parameters (cmpy/models/anderson.py:60-77,147-158);
    the hopping sign width is 0 like the reference."""
    mu = u / 2 if mu is None else mu
    eps_bath = np.atleast_1d(np.asarray(eps_bath, dtype=np.float64))
    v = np.atleast_1d(np.asarray(v, dtype=np.float64))
    nb = len(eps_bath)
    uu = np.append(u, np.zeros(nb)).astype(np.float64)
    eps = np.append(eps_imp - mu, eps_bath).astype(np.float64)
    bonds = [(0, j + 1, float(v[j])) for j in range(nb)]
    return eps, uu, bonds, 0


def coo_heisenberg(states, pairs):
    """HeisenbergModel._hamiltonian_data with per-pair couplings (cmpy/models/heisenberg.py:19-40):
    per state, per directed pair (pos1, pos2, j, jz): diagonal (sign*0.25)*jz always, and
    (0.25*j)/2 to the flipped state when the bits differ."""
    states = np.asarray(states, dtype=np.int64)
    D = len(states)
    per_state = []
    for p1, p2, j, jz in pairs:
        b1 = (states >> p1) & 1
        b2 = (states >> p2) & 1
        sign = np.where(b1 == b2, 1.0, -1.0)
        diag = (sign * 0.25) * jz
        differ = b1 != b2
        s2 = states ^ (1 << p1) ^ (1 << p2)
        idx2 = np.searchsorted(states, s2)
        off = np.full(D, (0.25 * j) / 2)
        per_state.append((diag, differ, idx2, off))
    rows, cols, vals = [], [], []
    ar = np.arange(D, dtype=np.int64)
    # emission order is state-major: build an index key (state, pair, sub) and sort
    keys, r_, c_, v_ = [], [], [], []
    P = len(pairs)
    for q, (diag, differ, idx2, off) in enumerate(per_state):
        keys.append(ar * (2 * P) + 2 * q)
        r_.append(ar)
        c_.append(ar)
        v_.append(diag)
        sel = np.nonzero(differ)[0]
        keys.append(sel * (2 * P) + 2 * q + 1)
        r_.append(sel)
        c_.append(idx2[sel])
        v_.append(off[sel])
    key = np.concatenate(keys)
    order = np.argsort(key, kind="stable")
    return (np.concatenate(r_)[order].astype(np.int64), np.concatenate(c_)[order].astype(np.int64),
            np.concatenate(v_)[order].astype(np.float64))


def heisenberg_pairs(neighbors, j=1.0, jz=None):
    """Directed pairs in emission order (heisenberg.py:20-24); j, jz scalars or (N,N) arrays."""
    jz = j if jz is None else jz
    get = lambda c, a, b: float(c) if np.ndim(c) == 0 else float(np.asarray(c)[a, b])
    return [(p1, int(p2), get(j, p1, p2), get(jz, p1, p2)) for p1 in range(len(neighbors)) for p2 in neighbors[p1]]


# ---- operators on vectors -------------------------------------------------------------------


def triplet_matvec(n, rows, cols, vals, x):
    """HamiltonOperator._matvec: y[col] += val * x[row] in triplet order
    (cmpy/operators.py:626-630). np.add.at accumulates sequentially, like the loop."""
    y = np.zeros(n, dtype=np.result_type(np.float64, np.asarray(x).dtype))
    np.add.at(y, cols, np.asarray(vals) * np.asarray(x)[rows])
    return y


def csr_from_coo(n, rows, cols, vals):
    """scipy CSR of H (sums duplicates), i.e. HamiltonOperator.toarray's matrix (operators.py:632-635)."""
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n))


def dense_from_coo(n, rows, cols, vals):
    return csr_from_coo(n, rows, cols, vals).toarray()


def apply_fermion(up, dn, up_t, dn_t, pos, sigma, create, x, jw_sign=False):
    """c^dag / c of cmpy/operators.py:652-703 from sector (up, dn) into (up_t, dn_t). The dn
    variant indexes the target with the target's stride (the reference uses the source's);
    jw_sign adds (-1)^(same-spin electrons below pos [+ all up electrons for dn])."""
    up, dn, up_t, dn_t = (np.asarray(a, dtype=np.int64) for a in (up, dn, up_t, dn_t))
    x = np.asarray(x)
    op = 1 << pos
    nd, nd_t = len(dn), len(dn_t)
    out = np.zeros((len(up_t) * nd_t,) + x.shape[1:], dtype=x.dtype)
    low = op - 1
    if sigma == UP:
        for i, s in enumerate(up):
            if bool(s & op) != (not create):
                continue
            t = s ^ op
            j = np.searchsorted(up_t, t)
            sg = -1 if (jw_sign and bin(int(s) & low).count("1") % 2) else 1
            out[j * nd_t:(j + 1) * nd_t] = sg * x[i * nd:(i + 1) * nd]
    else:
        for i, s in enumerate(dn):
            if bool(s & op) != (not create):
                continue
            t = s ^ op
            j = np.searchsorted(dn_t, t)
            for u_idx, su in enumerate(up):
                par = bin(int(s) & low).count("1") + bin(int(su)).count("1")
                sg = -1 if (jw_sign and par % 2) else 1
                out[u_idx * nd_t + j] = sg * x[u_idx * nd + i]
    return out


# ---- ground state and Green's functions (cmpy/exactdiag.py) -----------------------------------


def ground_state_dense(H):
    w, v = np.linalg.eigh(H)
    i = int(np.argmin(w))
    return w[i], v[:, i]


def gf_lehmann_thermal(sector_dense, sector_states_fn, num_sites, z, beta, pos=0, sigma=UP, jw_sign=False):
    """Thermal Lehmann G(z) (cmpy/exactdiag.py:110-245): GreensFunctionMeasurement over all
    (n_up, n_dn) sectors that have an upper sector. sector_dense(n_up, n_dn) -> dense H;
    sector_states_fn(n) -> states. Returns (gf, occ, occ_double, gs_energy)."""
    z = np.asarray(z, dtype=np.complex128)
    part, gs_energy = 0.0, np.inf
    gf = np.zeros_like(z)
    occ = 0.0
    occ2 = 0.0
    cache = {}

    def solve(nu, nd):
        if (nu, nd) not in cache:
            cache[(nu, nd)] = np.linalg.eigh(sector_dense(nu, nd))
        return cache[(nu, nd)]

    for n_up in range(num_sites + 1):
        for n_dn in range(num_sites + 1):
            tgt = (n_up + 1, n_dn) if sigma == UP else (n_up, n_dn + 1)
            if tgt[0] > num_sites or tgt[1] > num_sites:
                continue
            w, v = solve(n_up, n_dn)
            wp, vp = solve(*tgt)
            emin = w.min()
            factor = 1.0
            if emin < gs_energy:
                factor = np.exp(-beta * (gs_energy - emin))
                gs_energy = emin
            e0 = gs_energy
            part = part * factor + np.sum(np.exp(-beta * (w - e0)))
            gf *= factor
            up, dn = sector_states_fn(n_up), sector_states_fn(n_dn)
            up_t, dn_t = sector_states_fn(tgt[0]), sector_states_fn(tgt[1])
            cv = apply_fermion(up, dn, up_t, dn_t, pos, sigma, True, v, jw_sign)
            ov = np.abs(vp.T.conj() @ cv) ** 2
            if np.isfinite(beta):
                ew, ewp = np.exp(-beta * (w - e0)), np.exp(-beta * (wp - e0))
            else:
                ew, ewp = np.ones_like(w), np.ones_like(wp)
            for m in range(len(wp)):
                wts = ew + ewp[m]
                gf += np.sum(ov[m][None, :] * wts[None, :] / (z[:, None] - wp[m] + w[None, :]), axis=1)
            bw = np.exp(-beta * (w - e0))
            V = v.reshape(len(up), len(dn), -1)
            if sigma == UP:
                sel = ((up >> pos) & 1) == 1
                ov_occ = np.sum(np.abs(V[sel]) ** 2, axis=(0, 1))
            else:
                sel = ((dn >> pos) & 1) == 1
                ov_occ = np.sum(np.abs(V[:, sel]) ** 2, axis=(0, 1))
            occ = occ * factor + np.sum(bw * ov_occ)
            both = (((up[:, None] & dn[None, :]) >> pos) & 1) == 1
            occ2 = occ2 * factor + np.sum(bw * np.sum(np.abs(V[both]) ** 2, axis=0))
    return gf / part, occ / part, occ2 / part, gs_energy


def gf_zero_temperature_dense(H0, H_p, H_m, cdag_psi, c_psi, e0, z):
    """T=0 G(z) = sum_m |<m|c^dag|0>|^2/(z-E_m+E0) + sum_n |<n|c|0>|^2/(z+E_n-E0) by dense eigh."""
    z = np.asarray(z, dtype=np.complex128)
    g = np.zeros_like(z)
    if H_p is not None:
        w, v = np.linalg.eigh(H_p)
        amp = (v.T @ cdag_psi) ** 2
        g += np.sum(amp[None, :] / (z[:, None] - (w[None, :] - e0)), axis=1)
    if H_m is not None:
        w, v = np.linalg.eigh(H_m)
        amp = (v.T @ c_psi) ** 2
        g += np.sum(amp[None, :] / (z[:, None] + (w[None, :] - e0)), axis=1)
    return g


def lanczos_tridiag_dense(H, v0, m):
    """Lanczos coefficients with full reorthogonalisation in FP64 (a[m], b[m+1], ||v0||)."""
    n = H.shape[0]
    nrm = np.linalg.norm(v0)
    Q = np.zeros((n, m + 1))
    Q[:, 0] = v0 / nrm
    a = np.zeros(m)
    b = np.zeros(m + 1)
    for k in range(m):
        w = H @ Q[:, k]
        a[k] = Q[:, k] @ w
        w -= Q[:, : k + 1] @ (Q[:, : k + 1].T @ w)
        w -= Q[:, : k + 1] @ (Q[:, : k + 1].T @ w)
        b[k + 1] = np.linalg.norm(w)
        if b[k + 1] < 1e-12:
            return a[: k + 1], b[: k + 2], nrm
        Q[:, k + 1] = w / b[k + 1]
    return a, b, nrm


def tridiag_lowest(a, b):
    """Lowest eigenvalue of the tridiagonal (a, b[1:]) (scipy eigh_tridiagonal,
    as in cmpy/exactdiag.py:368-375)."""
    w = la.eigh_tridiagonal(np.asarray(a), np.asarray(b[1: len(a)]), eigvals_only=True, select="i",
                            select_range=(0, 0))
    return float(w[0])


# ---- real-time Green's functions: cmpy/exactdiag.py:248-316 ---------------------------------


def gf_time_dense(H_target: np.ndarray, start_vec: np.ndarray, e0: float, times, greater: bool) -> np.ndarray:
    """gf_greater (exactdiag.py:248-273) / gf_lesser (exactdiag.py:276-301) from the dense
    eigenpairs of the target sector: with phi = c^dag|gs> (greater) or c|gs> (lesser),
      greater: -i e^{i E0 t} <phi|e^{-iHt}|phi>,   lesser: +i e^{-i E0 t} <phi|e^{+iHt}|phi>.
    The reference evaluates e^{-+iHt} phi with scipy expm_multiply; the spectral sum is the
    same function."""
    w, V = np.linalg.eigh(H_target)
    amp = (V.T @ np.asarray(start_vec, dtype=np.float64)) ** 2
    t = np.asarray(times, dtype=np.float64)
    s = 1.0 if greater else -1.0
    phase = np.exp(-1j * s * np.outer(t, w - e0))
    return -1j * s * (phase @ amp)


def laplace_lin(times, gf_t, z) -> np.ndarray:
    """int_{t_0}^{t_last} e^{izt} g(t) dt of the piecewise-linear interpolant of g — the rule
    gftool.fourier.tt2z applies by default (tt2z_lin; gftool >= 0.10, pinned by cmpy's
    setup.cfg:30 / requirements.txt:11, absent here): per segment h e^{u t_j} [g_j phi2(uh) +
    g_{j+1} (phi1 - phi2)(uh)], u = iz, phi1(x) = (e^x-1)/x, phi2(x) = (e^x-1-x)/x^2."""
    t = np.asarray(times, dtype=np.float64)
    g = np.asarray(gf_t, dtype=np.complex128)
    z = np.asarray(z, dtype=np.complex128)
    u = 1j * z[:, None]
    h = np.diff(t)[None, :]
    x = u * h
    small = np.abs(x) < 0.25
    xs = np.where(small, 1.0, x)
    phi1 = np.where(small, 0, (np.exp(xs) - 1) / xs)
    phi2 = np.where(small, 0, (np.exp(xs) - 1 - xs) / xs**2)
    if np.any(small):
        a = np.zeros_like(x)
        b = np.zeros_like(x)
        fact1, fact2 = 1.0, 1.0
        for k in range(17):  # Taylor: phi1 = sum x^k/(k+1)!, phi2 = sum x^k/(k+2)!
            fact1 *= k + 1
            fact2 *= k + 2
            a = a + x**k / fact1
            b = b + x**k / fact2
        phi1 = np.where(small, a, phi1)
        phi2 = np.where(small, b, phi2)
    ej = np.exp(u * t[None, :-1])
    seg = h * ej * (g[None, :-1] * phi2 + g[None, 1:] * (phi1 - phi2))
    return seg.sum(axis=1)


# ---- G_ij: lehmann_full.py:19-97 ---------------------------------------------------------------


def _sector_dense(n_sites, desc, nu, nd):
    eps, u, bonds, width = desc
    up, dn = sector_states(n_sites, nu), sector_states(n_sites, nd)
    r, c, v = coo_fermion(up, dn, eps, u, bonds, width)
    return dense_from_coo(len(up) * len(dn), r, c, v), up, dn


def greens_lehmann_draft(n_sites, desc, z, beta, i, j, sigma=UP):
    """The reference's draft greens_lehmann (lehmann_full.py:48-97) as written: the sector
    loop variable `i` shadows the site argument, so the annihilator acts on site = sector index
    (lehmann_full.py:67,88); the overlap is |<n|c_pos|m>|^2 (lehmann_full.py:20-21); the sum is
    not divided by the partition function. j does not enter."""
    z = np.asarray(z, dtype=np.complex128)
    gf = np.zeros_like(z)
    e0 = np.inf
    fillings = [(a, b) for a in range(n_sites + 1) for b in range(n_sites + 1)]
    for idx, (n_up, n_dn) in enumerate(fillings):
        up_t = n_up + 1 if sigma == UP else n_up
        dn_t = n_dn + 1 if sigma != UP else n_dn
        if up_t > n_sites or dn_t > n_sites:
            continue
        H, up, dn = _sector_dense(n_sites, desc, n_up, n_dn)
        Hp, upp, dnp = _sector_dense(n_sites, desc, up_t, dn_t)
        w, V = np.linalg.eigh(H)
        wp, Vp = np.linalg.eigh(Hp)
        min_energy = w.min()
        factor = 1.0
        if min_energy < e0:
            factor = np.exp(-beta * (e0 - min_energy))
            e0 = min_energy
        if factor != 1.0:
            gf *= factor
        pos = idx  # the shadowed loop variable
        if pos < n_sites:
            # c_pos |m> for every eigenvector m of the upper sector, projected on <n|
            c_m = apply_fermion(upp, dnp, up, dn, pos, sigma, False, Vp)
            ov = (V.T @ c_m) ** 2  # [n, m]
        else:
            ov = np.zeros((len(w), len(wp)))
        if np.isfinite(beta):
            en, em = np.exp(-beta * (w - e0)), np.exp(-beta * (wp - e0))
        else:
            en, em = np.ones_like(w), np.ones_like(wp)
        for m in range(len(wp)):
            for n in range(len(w)):
                gf += ov[n, m] * (en[n] + em[m]) / (z - wp[m] + w[n])
    return gf


def gf_offdiag_dense(n_sites, desc, z, beta, i, j, sigma=UP):
    """Thermal G_ij(z) = Z^-1 sum <n|c_i|m><m|c^dag_j|n> (e^{-beta E_n} + e^{-beta E_m}) /
    (z - E_m + E_n) over all sectors having an upper sector (the completed lehmann_full.py:19-45,
    normalised like GreensFunctionMeasurement, exactdiag.py:137-212)."""
    z = np.asarray(z, dtype=np.complex128)
    terms = []
    e0 = np.inf
    for n_up in range(n_sites + 1):
        for n_dn in range(n_sites + 1):
            up_t = n_up + 1 if sigma == UP else n_up
            dn_t = n_dn + 1 if sigma != UP else n_dn
            if up_t > n_sites or dn_t > n_sites:
                continue
            H, up, dn = _sector_dense(n_sites, desc, n_up, n_dn)
            Hp, upp, dnp = _sector_dense(n_sites, desc, up_t, dn_t)
            w, V = np.linalg.eigh(H)
            wp, Vp = np.linalg.eigh(Hp)
            ai = Vp.T @ apply_fermion(up, dn, upp, dnp, i, sigma, True, V)
            aj = Vp.T @ apply_fermion(up, dn, upp, dnp, j, sigma, True, V)
            terms.append((w, wp, ai * aj))
            e0 = min(e0, w.min())
    gf = np.zeros_like(z)
    part = 0.0
    for w, wp, ov in terms:
        en, em = np.exp(-beta * (w - e0)), np.exp(-beta * (wp - e0))
        part += en.sum()
        pole = wp[:, None] - w[None, :]
        coef = ov * (en[None, :] + em[:, None])
        gf += (coef.reshape(-1)[None, :] / (z[:, None] - pole.reshape(-1)[None, :])).sum(axis=1)
    return gf / part
