"""The device radix sort that rebuilds every CSR in insertion order (stable
LSD sort, one launch per 8-bit digit with a chained look-back over
8192-item tiles)
and the single-pass prefix scan behind row pointers and compactions:
keys and carried indices equal a stable host sort for sizes around the
2048-item tile, odd and even digit counts, 32- and 64-bit keys, and digits
that every key shares."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu

CASES = [
    # n, key_bits, wide, const_lo, const_hi
    (0, 8, 0, 0, 0),
    (1, 8, 0, 0, 0),
    (2, 3, 0, 0, 0),
    (2047, 8, 0, 0, 0),
    (2048, 9, 0, 0, 0),
    (2049, 16, 0, 0, 0),
    (6145, 24, 0, 0, 0),
    (4095, 12, 0, 0, 0),
    (4096, 12, 0, 0, 0),
    (4097, 13, 0, 0, 0),
    (8193, 24, 0, 0, 0),
    (8191, 14, 0, 0, 0),
    (16385, 24, 0, 0, 0),
    (100_003, 17, 0, 0, 0),
    (1_000_000, 24, 0, 0, 0),
    (1_000_000, 32, 0, 0, 0),
    (300_001, 24, 0, 8, 16),      # the middle digit is the same in every key
    (300_001, 20, 0, 0, 20),      # every key equal
    (70_000, 40, 1, 0, 0),
    (500_000, 64, 1, 0, 0),       # eight passes
    (500_000, 56, 1, 24, 40),     # odd count with shared digits
    (4_194_305, 22, 0, 0, 0),
]


@pytest.mark.parametrize("n,bits,wide,lo,hi", CASES)
def test_radix_sort_matches_stable_host_sort(vh, n, bits, wide, lo, hi):
    from vahana_gb300._lib import check, lib
    bad = C.c_uint64(99)
    check(lib().vg_selftest_sort(n, bits, wide, lo, hi, 1234 + n, C.byref(bad)))
    assert bad.value == 0


@pytest.mark.parametrize("n", [0, 1, 4095, 4096, 4097, 100_003, 3_000_001, 16_777_217])
@pytest.mark.parametrize("wide", [0, 1])
@pytest.mark.parametrize("in_place", [0, 1])
def test_scan_matches_host_prefix_sum(vh, n, wide, in_place):
    from vahana_gb300._lib import check, lib
    if wide and n > 4_000_000:
        pytest.skip("the 64-bit case is covered at 3e6 items")
    bad = C.c_uint64(99)
    check(lib().vg_selftest_scan(n, wide, in_place, 4321 + n, C.byref(bad)))
    assert bad.value == 0


def test_lookback_wait_gives_up_with_a_status(vh):
    """Failure detection without a GPU fault: a look-back scan whose first
    tile never publishes ends with status 0x5e02 instead of waiting forever
    (the bounded wait of every chained scan and sort pass), and the context
    stays usable for the next scan."""
    from vahana_gb300._lib import check, lib
    status = C.c_int(0)
    ms = C.c_double(-1.0)
    check(lib().vg_selftest_scan_timeout(C.byref(status), C.byref(ms)))
    assert status.value == 0x5e02
    assert 0.0 < ms.value < 120_000.0
    bad = C.c_uint64(99)
    check(lib().vg_selftest_scan(3_000_001, 0, 0, 77, C.byref(bad)))
    assert bad.value == 0
