"""Addresses and occupation bitstrings (python/ffsim/states/bitstring.py):
every representation, spinful and spinless, against the reference's own code
(golden vectors) and its documented example."""

from __future__ import annotations

import numpy as np
import pytest


def test_documented_example():
    """norb=3, nelec=(2, 1): bitstring.py:178-200 lists these values."""
    import ffsim_gb300 as f

    assert f.addresses_to_strings(range(5), 3, (2, 1)) == [11, 19, 35, 13, 21]
    assert f.addresses_to_strings(range(5), 3, (2, 1), bitstring_type=f.BitstringType.STRING) == [
        "001011", "010011", "100011", "001101", "010101"]
    np.testing.assert_array_equal(f.strings_to_addresses([11, 19, 35, 13, 21], 3, (2, 1)), np.arange(5))


@pytest.mark.parametrize("tag, norb, nelec", [("s", 5, (2, 3)), ("l", 6, 3)])
def test_golden(golden, tag, norb, nelec):
    import ffsim_gb300 as f

    addrs = golden[f"bits{tag}_addrs"]
    for t in f.BitstringType:
        res = f.addresses_to_strings(addrs, norb, nelec, bitstring_type=t)
        np.testing.assert_array_equal(np.asarray(res), golden[f"bits{tag}_{t.name}"])
        if isinstance(nelec, tuple):
            a, b = f.addresses_to_strings(addrs, norb, nelec, concatenate=False, bitstring_type=t)
            np.testing.assert_array_equal(np.asarray(a), golden[f"bits{tag}_{t.name}_a"])
            np.testing.assert_array_equal(np.asarray(b), golden[f"bits{tag}_{t.name}_b"])
        back = f.strings_to_addresses(res, norb, nelec)
        assert back.dtype == np.int64
        np.testing.assert_array_equal(back, golden[f"bits{tag}_{t.name}_back"])


def test_conversions_and_errors():
    import ffsim_gb300 as f
    from ffsim_gb300 import bitstring as b

    assert b.convert_bitstring_type(["0101"], f.BitstringType.STRING, f.BitstringType.INT, 4) == [5]
    np.testing.assert_array_equal(b.convert_bitstring_type([5], f.BitstringType.INT, f.BitstringType.BIT_ARRAY, 4),
                                  [[False, True, False, True]])
    assert b.restrict_bitstrings([0b1101], [0, 2], f.BitstringType.INT) == [0b11]
    assert f.bitstring_to_occupied_orbitals(0b10110) == [1, 2, 4]
    assert len(f.strings_to_addresses([], 4, (2, 2))) == 0
    with pytest.raises(TypeError):
        b.convert_bitstring_type([1], "int", f.BitstringType.INT, 3)
    with pytest.raises(ValueError):
        f.strings_to_addresses([0b111], 4, 2)
