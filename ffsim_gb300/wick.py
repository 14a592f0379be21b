"""Wick's theorem on Slater determinants (python/ffsim/states/wick.py): the
expectation of a product of one-body operators O_i = sum M_i[p, q] a+_p a_q,
from the determinant's one-body density matrix alone.  Host arithmetic."""

from __future__ import annotations

import itertools
import string

import numpy as np


def expectation_one_body_product(one_rdm: np.ndarray, one_body_tensors) -> complex:
    """<psi| O_1 O_2 ... O_k |psi> for a Slater determinant with 1-RDM
    rho[p, q] = <a+_p a_q>, in spin orbitals (wick.py:15-94).

    Wick's theorem sums over the ways to pair each creator c_i with an
    annihilator a_j: a pair is rho[p_i, q_j] when the creator comes first in
    the operator string and (1 - rho)[p_i, q_j] when the annihilator does, and
    each pairing carries (-1) to the number of crossing pairs."""
    k = len(one_body_tensors)
    if not k:
        return 1.0
    n = one_rdm.shape[0]
    anti = np.eye(n) - one_rdm
    letters = string.ascii_letters
    cre = [letters[2 * i] for i in range(k)]
    ann = [letters[2 * i + 1] for i in range(k)]
    ops = ",".join(c + a for c, a in zip(cre, ann))
    total = 0.0
    for perm in itertools.permutations(range(k)):
        # positions in c_1 a_1 c_2 a_2 ...: creator i at 2i, annihilator j at 2j + 1
        arcs = [tuple(sorted((2 * i, 2 * perm[i] + 1))) for i in range(k)]
        crossings = sum(1 for (l1, r1), (l2, r2) in itertools.combinations(arcs, 2)
                        if l1 < l2 < r1 < r2 or l2 < l1 < r2 < r1)
        pairs = [one_rdm if i <= perm[i] else anti for i in range(k)]
        subs = ",".join(cre[i] + ann[perm[i]] for i in range(k))
        total += (-1) ** crossings * np.einsum(f"{ops},{subs}->", *one_body_tensors, *pairs, optimize=True)
    return total


def expectation_one_body_power(one_rdm: np.ndarray, one_body_tensor: np.ndarray, power: int = 1) -> complex:
    """<psi| O^k |psi> for a Slater determinant (wick.py:97-132)."""
    return expectation_one_body_product(one_rdm, [one_body_tensor] * power)
