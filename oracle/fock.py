"""ORACLE (test infrastructure, not product code): the objects of a two-site DMRG step
expanded into the full Fock space of a short chain, where the Hamiltonian is applied as
plain second-quantised operators.

This checker shares nothing with the product's task compiler or with the CPU oracle's
executor. From the MPS tensors (TensorT storage, read back from the product) and the
current sector dimensions alone it builds

  * the left renormalised states of boundary b as explicit many-electron vectors, by
    the left-to-right spin coupling of TensorT (CheMPS2/TensorT.cpp:38-110: block
    (NL, 2SL, IL) -> (NR, 2SR, IR), the site's spin coupled to the left spin), with
    Clebsch-Gordan coefficients;
  * the right completions of boundary b: for every right-block state the vector over
    the sites b .. L-1 that completes it to the total state (summed over the total
    state's M components);
  * the embedding P of the two-site object (CheMPS2/Sobject.cpp:36-145: blocks
    (NL, 2SL, IL, N1, N2, 2J, NR, 2SR, IR), the two sites coupled to 2J first, then 2SL
    and 2J to 2SR), so that P x is the many-electron state of a two-site vector x;
  * H = sum_ij T_ij E_ij + 1/2 sum_ijkl V_ijkl (E_ik E_jl - delta_jk E_il) + Econst on
    the 4^L configurations, V in physics notation V_ijkl = (ik|jl)
    (CheMPS2/include/chemps2/FourIndex.h:30-32), E_pq = sum_sigma a+_p,sigma a_q,sigma
    with Jordan-Wigner signs.

The effective Hamiltonian of the step is then Q^T H Q, Q = P with its columns
normalised; the product's Heff, its diagonal, Join and Split are compared against it.
Conventions: spin-orbital modes ordered site by site, up before down; the local states
of a site are |0>, a+_up|0>, a+_down|0>, a+_up a+_down|0>; Clebsch-Gordan coefficients
in the Condon-Shortley convention with the left spin first. Sizes: 4^L amplitudes per
vector, meant for L <= 8.
"""
from __future__ import annotations

import math
from functools import lru_cache

import numpy as np

# ---------------------------------------------------------------- Clebsch-Gordan


@lru_cache(maxsize=None)
def cg(j1, m1, j2, m2, J, M):
    """<j1 m1 j2 m2 | J M>, every argument twice the (half-)integer it stands for."""
    if m1 + m2 != M or abs(m1) > j1 or abs(m2) > j2 or abs(M) > J:
        return 0.0
    if not (abs(j1 - j2) <= J <= j1 + j2) or (j1 + j2 + J) % 2:
        return 0.0
    if (j1 + m1) % 2 or (j2 + m2) % 2 or (J + M) % 2:
        return 0.0
    f = math.factorial

    def h(x):  # x is twice an integer
        return x // 2

    pre = (J + 1) * f(h(J + j1 - j2)) * f(h(J - j1 + j2)) * f(h(j1 + j2 - J)) / f(h(j1 + j2 + J) + 1)
    pre *= f(h(J + M)) * f(h(J - M)) * f(h(j1 - m1)) * f(h(j1 + m1)) * f(h(j2 - m2)) * f(h(j2 + m2))
    s = 0.0
    for k in range(0, h(j1 + j2 - J) + 1):
        a = [k, h(j1 + j2 - J) - k, h(j1 - m1) - k, h(j2 + m2) - k, h(J - j2 + m1) + k, h(J - j1 - m2) + k]
        if min(a) < 0:
            continue
        d = 1
        for v in a:
            d *= f(v)
        s += (-1) ** k / d
    return math.sqrt(pre) * s


# ---------------------------------------------------------------- local states
# local state code: 0 empty, 1 up, 2 down, 3 up+down
def local_states(n):
    """[(2s, 2m, code)] of a site with n electrons."""
    if n == 0:
        return [(0, 0, 0)]
    if n == 2:
        return [(0, 0, 3)]
    return [(1, 1, 1), (1, -1, 2)]


# ---------------------------------------------------------------- sectors and blocks
def sector_dims(rows):
    """{(N, 2S, I): current dim} from (N, 2S, I, fci, cur) rows, dims > 0 only."""
    return {(int(r[0]), int(r[1]), int(r[2])): int(r[4]) for r in rows if int(r[4]) > 0}


def mps_blocks(left, right, site_irrep, data):
    """Blocks of one TensorT in storage order: left sectors (N, 2S, I) ascending, then
    NR = NL, NL+1, NL+2 and for NL+1 the right spin 2SL-1 before 2SL+1; each block
    dim_left x dim_right, column-major. Returns {(NL,SL,IL,NR,SR,IR): array}."""
    out = {}
    off = 0
    for (nl, sl, il) in sorted(left):
        dl = left[(nl, sl, il)]
        for nr in (nl, nl + 1, nl + 2):
            tj = 1 if nr == nl + 1 else 0
            for sr in range(sl - tj, sl + tj + 1, 2):
                if sr < 0:
                    continue
                ir = il ^ site_irrep if nr == nl + 1 else il
                dr = right.get((nr, sr, ir), 0)
                if dr <= 0:
                    continue
                out[(nl, sl, il, nr, sr, ir)] = data[off:off + dl * dr].reshape((dl, dr), order="F")
                off += dl * dr
    if off != len(data):
        raise ValueError(f"tensor length {len(data)} differs from its blocks ({off})")
    return out


def sobject_blocks(left, right, irrep1, irrep2):
    """Blocks of the two-site object in CheMPS2/Sobject.cpp:36-145 order:
    [((NL,SL,IL,N1,N2,TJ,NR,SR,IR), dim_left, dim_right)]."""
    blocks = []
    for (nl, sl, il) in sorted(left):
        dl = left[(nl, sl, il)]
        for n1 in range(3):
            for n2 in range(3):
                tjmin = 1 if (n1 == 1) != (n2 == 1) else 0
                tjmax = (1 if n1 == 1 else 0) + (1 if n2 == 1 else 0)
                for tj in range(tjmin, tjmax + 1, 2):
                    nr = nl + n1 + n2
                    ir = il ^ (irrep1 if n1 == 1 else 0) ^ (irrep2 if n2 == 1 else 0)
                    for sr in range(sl - tj, sl + tj + 1, 2):
                        if sr < 0:
                            continue
                        dr = right.get((nr, sr, ir), 0)
                        if dr > 0:
                            blocks.append(((nl, sl, il, n1, n2, tj, nr, sr, ir), dl, dr))
    return blocks


# ---------------------------------------------------------------- the chain
class FockChain:
    """The MPS of a chain of L sites: tensors[site] (TensorT storage) with sectors[b]
    ({(N, 2S, I): dim} for boundaries b = 0 .. L), the orbital irreps and the total
    (N, 2S, I)."""

    def __init__(self, L, irreps, sectors, tensors, total):
        self.L = L
        self.irreps = [int(i) for i in irreps]
        self.sectors = sectors
        self.total = total
        self.T = [mps_blocks(sectors[k], sectors[k + 1], self.irreps[k], np.asarray(tensors[k], dtype=np.float64))
                  for k in range(L)]
        self._left = {0: {(0, 0, 0): np.ones((1, 1, 1))}}
        self._right = {}

    # left states of boundary b: {(N, 2S, I): array (dim, 2S + 1, 4^b)}
    def left(self, b):
        if b in self._left:
            return self._left[b]
        prev = self.left(b - 1)
        site = b - 1
        nconf = 4 ** (b - 1)
        # every sector of the boundary, also one that no block of the site feeds (its
        # states are then zero vectors)
        out = {k: np.zeros((dim, k[1] + 1, nconf, 4)) for k, dim in self.sectors[b].items()}
        for (nl, sl, il, nr, sr, ir), T in self.T[site].items():
            Lv = prev[(nl, sl, il)]
            dst = out[(nr, sr, ir)]
            for (s2, m2, code) in local_states(nr - nl):
                for mri, mr in enumerate(range(-sr, sr + 1, 2)):
                    ml = mr - m2
                    if abs(ml) > sl:
                        continue
                    c = cg(sl, ml, s2, m2, sr, mr)
                    if c == 0.0:
                        continue
                    dst[:, mri, :, code] += c * (T.T @ Lv[:, (ml + sl) // 2, :])
        out = {k: v.reshape(v.shape[0], v.shape[1], nconf * 4) for k, v in out.items()}
        self._left[b] = out
        return out

    # right completions of boundary b: {(N, 2S, I): array (dim, 2S + 1, 4^(L - b))}
    def right(self, b):
        if b in self._right:
            return self._right[b]
        if b == self.L:
            # every M component of the total spin multiplet, each with weight one: with
            # this completion the squared norm of a right state of spin SR is 2SR + 1 at
            # every boundary (the symmetric normalisation of the two-site object)
            n, s2, i = self.total
            self._right[b] = {(n, s2, i): np.ones((1, s2 + 1, 1))}
            return self._right[b]
        nxt = self.right(b + 1)
        site = b
        nconf = 4 ** (self.L - b - 1)
        out = {k: np.zeros((dim, k[1] + 1, 4, nconf)) for k, dim in self.sectors[b].items()}
        for (nl, sl, il, nr, sr, ir), T in self.T[site].items():
            R = nxt.get((nr, sr, ir))
            if R is None:
                continue
            dst = out[(nl, sl, il)]
            for (s2, m2, code) in local_states(nr - nl):
                for mli, ml in enumerate(range(-sl, sl + 1, 2)):
                    mr = ml + m2
                    if abs(mr) > sr:
                        continue
                    c = cg(sl, ml, s2, m2, sr, mr)
                    if c == 0.0:
                        continue
                    dst[:, mli, code, :] += c * (T @ R[:, (mr + sr) // 2, :])
        out = {k: v.reshape(v.shape[0], v.shape[1], 4 * nconf) for k, v in out.items()}
        self._right[b] = out
        return out

    def state(self, all_m=False):
        """The MPS as one many-electron vector (4^L amplitudes): its M = S component, or
        with all_m the sum of all M components of the multiplet (what the two-site
        embedding below produces)."""
        L = self.left(self.L)
        n, s2, i = self.total
        v = L[(n, s2, i)][0]
        return v.sum(axis=0) if all_m else v[s2, :].copy()


class TwoSite:
    """The embedding of the two-site object at sites (index, index + 1) of a chain."""

    def __init__(self, chain: FockChain, index: int):
        self.c = chain
        self.index = index
        L = chain.L
        self.blocks = sobject_blocks(chain.sectors[index], chain.sectors[index + 2], chain.irreps[index],
                                     chain.irreps[index + 1])
        self.offsets = np.concatenate([[0], np.cumsum([dl * dr for _, dl, dr in self.blocks])]).astype(np.int64)
        self.size = int(self.offsets[-1])
        self.nl = 4 ** index
        self.nr = 4 ** (L - index - 2)
        self.Lb = chain.left(index)
        self.Rb = chain.right(index + 2)
        # (block, ML, m1, m2, MR) terms with their coupling coefficients
        self.terms = []
        for kb, ((nl, sl, il, n1, n2, tj, nr, sr, ir), dl, dr) in enumerate(self.blocks):
            for (a1, m1, c1) in local_states(n1):
                for (a2, m2, c2) in local_states(n2):
                    mj = m1 + m2
                    w12 = cg(a1, m1, a2, m2, tj, mj)
                    if w12 == 0.0:
                        continue
                    for ml in range(-sl, sl + 1, 2):
                        mr = ml + mj
                        if abs(mr) > sr:
                            continue
                        w = w12 * cg(sl, ml, tj, mj, sr, mr)
                        if w != 0.0:
                            self.terms.append((kb, (ml + sl) // 2, c1, c2, (mr + sr) // 2, w))
        # Blocks whose spins violate the triangle rule (2SL, 2J, 2SR) exist in the block list
        # (the reference's loop takes 2SR from 2SL - 2J to 2SL + 2J) but have no physical
        # state: P maps them to zero. `physical` marks the entries of the other blocks.
        self.physical = np.zeros(self.size, dtype=bool)
        for kb, ((nl, sl, il, n1, n2, tj, nr, sr, ir), dl, dr) in enumerate(self.blocks):
            if abs(sl - tj) <= sr <= sl + tj:
                self.physical[self.offsets[kb]:self.offsets[kb + 1]] = True
        # squared norms of the columns of P, block by block (one value per right index)
        self.norm2 = np.zeros(self.size)
        for kb, ((nl, sl, il, n1, n2, tj, nr, sr, ir), dl, dr) in enumerate(self.blocks):
            R = self.Rb[(nr, sr, ir)]
            nb = np.einsum("bmc,bmc->b", R, R)  # sum over MR of |R_b,MR|^2
            o = self.offsets[kb]
            self.norm2[o:o + dl * dr] = np.tile(nb, (dl, 1)).ravel(order="F")

    def block(self, x, kb):
        _, dl, dr = self.blocks[kb]
        o = self.offsets[kb]
        return x[o:o + dl * dr].reshape((dl, dr), order="F")

    def embed(self, x):
        """P x: the many-electron state of two-site vector x (coefficients as stored)."""
        psi = np.zeros((self.nl, 4, 4, self.nr))
        for kb, mli, c1, c2, mri, w in self.terms:
            lab = self.blocks[kb][0]
            Lv = self.Lb[lab[0:3]][:, mli, :]
            R = self.Rb[lab[6:9]][:, mri, :]
            psi[:, c1, c2, :] += w * (Lv.T @ self.block(x, kb) @ R)
        return psi.ravel()

    def project(self, psi):
        """P^T psi."""
        P = psi.reshape(self.nl, 4, 4, self.nr)
        x = np.zeros(self.size)
        for kb, mli, c1, c2, mri, w in self.terms:
            lab = self.blocks[kb][0]
            Lv = self.Lb[lab[0:3]][:, mli, :]
            R = self.Rb[lab[6:9]][:, mri, :]
            _, dl, dr = self.blocks[kb]
            o = self.offsets[kb]
            x[o:o + dl * dr] += w * (Lv @ P[:, c1, c2, :] @ R.T).ravel(order="F")
        return x


# ---------------------------------------------------------------- the Hamiltonian
class FockHamiltonian:
    """H on the 4^L configurations of the chain (site 0 the most significant base-4 digit)."""

    def __init__(self, tmat, vmat, econst=0.0):
        import scipy.sparse as sp

        L = tmat.shape[0]
        self.L = L
        dim = 4 ** L
        conf = np.arange(dim)
        digits = np.stack([(conf // 4 ** (L - 1 - k)) % 4 for k in range(L)], axis=1)  # [conf, site]
        occ = np.zeros((dim, 2 * L), dtype=np.int64)  # mode 2k + sigma
        occ[:, 0::2] = digits & 1
        occ[:, 1::2] = (digits >> 1) & 1
        before = np.cumsum(occ, axis=1) - occ  # occupied modes before each mode
        weights = np.array([4 ** (L - 1 - k) for k in range(L)])
        E = {}
        for p in range(L):
            for q in range(L):
                rows, cols, vals = [], [], []
                for sig in (0, 1):
                    mp, mq = 2 * p + sig, 2 * q + sig
                    bit = 1 if sig == 0 else 2
                    ok = occ[:, mq] == 1
                    sign = (-1.0) ** before[:, mq]
                    if p == q:
                        r = conf[ok]
                        rows.append(r)
                        cols.append(r)
                        vals.append(np.ones(r.size))
                        continue
                    # after a_q: occupation minus mode q; a+_p needs mode p empty
                    ok2 = ok & (occ[:, mp] == 0)
                    src = conf[ok2]
                    nb = before[ok2, mp] - (1 if mq < mp else 0)
                    sgn = sign[ok2] * (-1.0) ** nb
                    dst = src - bit * weights[q] + bit * weights[p]
                    rows.append(dst)
                    cols.append(src)
                    vals.append(sgn)
                E[(p, q)] = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                                          shape=(dim, dim))
        self.E = E
        self.T = np.asarray(tmat, dtype=np.float64)
        self.V = np.asarray(vmat, dtype=np.float64)
        self.econst = float(econst)
        # T'_il = T_il - 1/2 sum_j V_ijjl
        self.Tp = self.T - 0.5 * np.einsum("ijjl->il", self.V)
        self.Vr = self.V.transpose(0, 2, 1, 3).reshape(L * L, L * L)  # [(i,k),(j,l)]

    def apply(self, v):
        """H v for one vector (4^L) or the columns of a matrix (4^L x k)."""
        L = self.L
        W = np.stack([self.E[(j, l)] @ v for j in range(L) for l in range(L)])  # [(j,l), conf(, k)]
        U = np.tensordot(self.Vr, W, axes=(1, 0))  # [(i,k), conf(, k)]
        out = self.econst * v
        for i in range(L):
            for k in range(L):
                out = out + self.E[(i, k)] @ (self.Tp[i, k] * v + 0.5 * U[i * L + k])
        return out


# ---------------------------------------------------------------- the effective Hamiltonian
def heff(ts: TwoSite, H: FockHamiltonian, x):
    """Q^T H Q x for a two-site vector x in the stored (symmetric) normalisation, Q = P
    with unit columns; entries of blocks without a physical state are zero in and out."""
    s = np.where(ts.physical, 1.0 / np.sqrt(np.where(ts.norm2 > 0, ts.norm2, 1.0)), 0.0)
    return s * ts.project(H.apply(ts.embed(s * x)))


def heff_columns(ts: TwoSite, H: FockHamiltonian, cols):
    """The columns `cols` of Q^T H Q (one H application on all of them at once)."""
    s = np.where(ts.physical, 1.0 / np.sqrt(np.where(ts.norm2 > 0, ts.norm2, 1.0)), 0.0)
    psi = np.stack([ts.embed(s * np.eye(1, ts.size, j).ravel()) for j in cols], axis=1)
    hp = H.apply(psi)
    return np.stack([s * ts.project(hp[:, c]) for c in range(len(cols))], axis=1)


def joined_state(ts: TwoSite, x):
    """The many-electron state of a two-site vector in the stored normalisation."""
    s = np.where(ts.physical, 1.0 / np.sqrt(np.where(ts.norm2 > 0, ts.norm2, 1.0)), 0.0)
    return ts.embed(s * x)


def two_rdm_a(H: FockHamiltonian, psi):
    """The spin-summed 2-RDM A_ijkl = sum_{sigma,tau} <a+_i,s a+_j,t a_l,t a_k,s> of the
    state psi (normalised here), from the E operators of H: <E_ik E_jl> - delta_jk <E_il>."""
    L = H.L
    psi = psi / np.sqrt(psi @ psi)
    Ev = {(p, q): H.E[(p, q)] @ psi for p in range(L) for q in range(L)}
    A = np.zeros((L, L, L, L))
    one = np.array([[psi @ Ev[(i, l)] for l in range(L)] for i in range(L)])
    for i in range(L):
        for k in range(L):
            left = Ev[(k, i)]  # (E_ki psi) = (E_ik^T psi)
            for j in range(L):
                for l in range(L):
                    A[i, j, k, l] = left @ Ev[(j, l)]
    for j in range(L):
        A[:, j, j, :] -= one
    return A
