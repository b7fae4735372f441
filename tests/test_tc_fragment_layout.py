"""Index arithmetic of the plane-wave tensor-core kernel's spectra fragments, restated.

tc_prep_kernel (f_number_gb300/csrc/fnum_kernels.cu) writes fragment i of the buffer
tc_B for angle pass ap, bin kk, element group s, n-tile j and lane, with
    i = (((ap * K + kk) * S + s) * nt + j) * 32 + lane,
nt n-tiles of 4 angles per pass (3 or 4).  pw_tc_tile reads, for the pass starting at
angle a0, the element pass starting at e0, bin k, k-step s and n-tile j,
    (a0 / 4nt) K S 32nt + (e0 / 8) 32nt + (k - k_lb) S 32nt + s 32nt + j 32 + lane.
These must name the same fragment, that fragment must hold the angles and elements the
tile multiplies, and every read must stay inside the buffer the plan allocates (the
larger of the 12- and 16-angle layouts, S = ceil(ne / 8) + TC_KS - 1 groups).  No GPU."""
import itertools

import pytest

TC_KS = 2    # k-steps (groups of 8 elements) per element pass
TC_EP = 16   # elements per element pass


def ntiles_for(na):
    """Passes of 16 angles where they take fewer passes than passes of 12."""
    return 4 if (na + 15) // 16 < (na + 11) // 12 else 3


def groups(ne):
    return (ne + 7) // 8 + TC_KS - 1


def buffer_len(na, K, ne):
    S = groups(ne)
    return max(((na + 4 * nt - 1) // (4 * nt)) * K * S * 32 * nt for nt in {3, ntiles_for(na)})


def prep_decompose(i, K, S, nt):
    lane = i & 31
    r = i >> 5
    j = r % nt
    r //= nt
    s = r % S
    r //= S
    kk = r % K
    ap = r // K
    return ap, kk, s, j, lane


def tile_address(a0, e0, k, k_lb, s, j, lane, K, S, nt):
    NB = 32 * nt
    Bp = (a0 // (4 * nt)) * K * S * NB
    Bpe = Bp + (e0 >> 3) * NB + lane
    Bk = Bpe + (k - k_lb) * S * NB
    return Bk + s * NB + j * 32


def test_pass_width_rule():
    assert [n for n in range(1, 65) if ntiles_for(n) == 4] == list(range(13, 17)) + list(range(25, 33)) + \
        list(range(37, 65))
    for na in range(1, 200):
        nt = ntiles_for(na)
        assert (na + 4 * nt - 1) // (4 * nt) <= (na + 11) // 12   # never more passes


@pytest.mark.parametrize("na,ne", [(11, 128), (13, 45), (31, 24), (36, 16), (49, 20), (5, 192), (64, 9)])
def test_tile_reads_the_fragments_the_prep_writes(na, ne):
    K, k_lb = 7, 3
    S = groups(ne)
    n_buf = buffer_len(na, K, ne)
    for nt in sorted({3, ntiles_for(na)}):   # the plan's passes, and the derivative kernel's 12-angle passes
        n_ap = (na + 4 * nt - 1) // (4 * nt)
        assert n_ap * K * S * nt * 32 <= n_buf   # the prep writes inside the buffer
        # element passes: from a multiple of 8 up to the last element, in steps of 16
        e_passes = [e0 for e0 in range(0, ne, TC_EP)] + [e0 for e0 in range(8, ne, TC_EP)]
        for a0, e0, k, s, j, lane in itertools.product(range(0, na, 4 * nt), e_passes, range(k_lb, k_lb + K),
                                                       range(TC_KS), range(nt), (0, 5, 31)):
            addr = tile_address(a0, e0, k, k_lb, s, j, lane, K, S, nt)
            assert 0 <= addr < n_buf
            ap, kk, sg, jj, ln = prep_decompose(addr, K, S, nt)
            assert (ap, kk, sg, jj, ln) == (a0 // (4 * nt), k - k_lb, (e0 >> 3) + s, j, lane)
            # the fragment's angle and elements: lane (g, q) holds angle ap 4nt + 4j + g / 2 and
            # elements 8 sg + 2q + t, t = 0, 1 -- the tile's angle a0 + 4j + g / 2 and its
            # k-step's elements e0 + 8s + 2q + t
            g, q = ln >> 2, ln & 3
            assert ap * 4 * nt + 4 * jj + (g >> 1) == a0 + 4 * j + (g >> 1)
            assert 8 * sg + 2 * q == (e0 & ~7) + 8 * s + 2 * q
