"""Occupation bitstrings and state-vector addresses (python/ffsim/states/bitstring.py).

The address of a spinful configuration is ``addr_a * dim_b + addr_b``, where
a sector address is the rank of its bitstring among the ascending integers
with the same number of set bits.  Bitstrings come as Python ints, '0'/'1'
strings (highest orbital first) or boolean arrays (highest orbital first);
concatenated spinful bitstrings put the beta bits above the alpha bits.
"""

from __future__ import annotations

import math
from enum import Enum, auto

import numpy as np

from ffsim_gb300.states import make_strings


class BitstringType(Enum):
    """Representation of bitstrings (python/ffsim/states/bitstring.py:24-45)."""

    STRING = auto()
    INT = auto()
    BIT_ARRAY = auto()


def _check_type(t, what: str) -> None:
    if not isinstance(t, BitstringType):
        raise TypeError(f"{what} must be ffsim.BitstringType.STRING, ffsim.BitstringType.INT, "
                        f"or ffsim.BitstringType.BIT_ARRAY. Got {t}.")


def convert_bitstring_type(strings, input_type: BitstringType, output_type: BitstringType, length: int):
    """Convert bitstrings between representations (bitstring.py:48-114)."""
    _check_type(input_type, "input_type")
    _check_type(output_type, "output_type")
    if input_type is output_type:
        return strings
    if input_type is BitstringType.STRING:
        ints = [int(s, base=2) for s in strings]
    elif input_type is BitstringType.BIT_ARRAY:
        ints = [sum(int(bit) << i for i, bit in enumerate(bits[::-1])) for bits in strings]
    else:
        ints = [int(s) for s in strings]
    if output_type is BitstringType.INT:
        return ints
    if output_type is BitstringType.STRING:
        return [f"{s:0{length}b}" for s in ints]
    if not ints:
        return np.empty((0, length), dtype=bool)
    return np.array([[(s >> i) & 1 for i in range(length - 1, -1, -1)] for s in ints], dtype=bool)


def restrict_bitstrings(strings, indices, bitstring_type: BitstringType):
    """Keep the bits at ``indices`` (lowest first) (bitstring.py:117-142)."""
    indices = list(indices)
    if bitstring_type is BitstringType.STRING:
        return ["".join(s[-1 - i] for i in indices[::-1]) for s in strings]
    if bitstring_type is BitstringType.INT:
        return [sum(((s >> index) & 1) << i for i, index in enumerate(indices)) for s in strings]
    return np.asarray(strings)[:, [-1 - i for i in indices[::-1]]]


def concatenate_bitstrings(strings_a, strings_b, bitstring_type: BitstringType, length: int):
    """Join alpha and beta bitstrings, beta bits above alpha (bitstring.py:145-170)."""
    if bitstring_type is BitstringType.STRING:
        return [s_b + s_a for s_a, s_b in zip(strings_a, strings_b)]
    if bitstring_type is BitstringType.INT:
        return [(s_b << length) + s_a for s_a, s_b in zip(strings_a, strings_b)]
    return np.concatenate([strings_b, strings_a], axis=1)


def addresses_to_strings(addresses, norb: int, nelec, concatenate: bool = True,
                         bitstring_type: BitstringType = BitstringType.INT):
    """Bitstrings of state-vector addresses (bitstring.py:173-263)."""
    addresses = np.asarray(addresses, dtype=np.int64)
    if isinstance(nelec, (int, np.integer)):
        ints = [int(s) for s in make_strings(norb, int(nelec))[addresses]]
        return convert_bitstring_type(ints, BitstringType.INT, bitstring_type, norb)
    n_alpha, n_beta = nelec
    idx_a, idx_b = np.divmod(addresses, math.comb(norb, n_beta))
    strings_a = convert_bitstring_type([int(s) for s in make_strings(norb, n_alpha)[idx_a]], BitstringType.INT,
                                       bitstring_type, norb)
    strings_b = convert_bitstring_type([int(s) for s in make_strings(norb, n_beta)[idx_b]], BitstringType.INT,
                                       bitstring_type, norb)
    if concatenate:
        return concatenate_bitstrings(strings_a, strings_b, bitstring_type, norb)
    return strings_a, strings_b


def _sector_addresses(norb: int, nocc: int, strings) -> np.ndarray:
    table = make_strings(norb, nocc)
    strings = np.asarray(strings, dtype=np.int64)
    addr = np.searchsorted(table, strings)
    if strings.size and (np.any(addr >= len(table)) or np.any(table[np.minimum(addr, len(table) - 1)] != strings)):
        raise ValueError(f"a bitstring does not have {nocc} of {norb} orbitals occupied")
    return addr.astype(np.int64)


def strings_to_addresses(strings, norb: int, nelec) -> np.ndarray:
    """State-vector addresses of bitstrings of any representation (bitstring.py:266-361)."""
    if not len(strings):
        return np.array([])
    if isinstance(strings, np.ndarray) and strings.ndim == 2:
        in_type = BitstringType.BIT_ARRAY
    elif isinstance(strings[0], str):
        in_type = BitstringType.STRING
    else:
        in_type = BitstringType.INT
    length = norb if isinstance(nelec, (int, np.integer)) else 2 * norb
    ints = convert_bitstring_type(strings, in_type, BitstringType.INT, length)
    if isinstance(nelec, (int, np.integer)):
        return _sector_addresses(norb, int(nelec), ints)
    n_alpha, n_beta = nelec
    mask = (1 << norb) - 1
    addr_a = _sector_addresses(norb, n_alpha, [s & mask for s in ints])
    addr_b = _sector_addresses(norb, n_beta, [s >> norb for s in ints])
    return addr_a * math.comb(norb, n_beta) + addr_b


def bitstring_to_occupied_orbitals(bitstring: int) -> list[int]:
    """The set bits of an integer bitstring, lowest first (bitstring.py:364-)."""
    out, i = [], 0
    while bitstring >> i:
        if (bitstring >> i) & 1:
            out.append(i)
        i += 1
    return out
