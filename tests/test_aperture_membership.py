"""The tensor-core plane-wave kernel decides aperture membership from the window
argument: element e is in the aperture of a voxel at x exactly when
u = |c_e - x| / L_side < 1, with L_left = x - lb[i_lb] and L_right = ub[i_ub] - x,
and a side without aperture counts as outside.  The index rule it replaced takes
e in [i_lb, emid) on the left and [emid, i_ub] on the right (emid = first element
with c_e >= x), i_lb = max(ceil(M + (x - h)/pitch), 0), i_ub = min(floor(M + (x + h)/pitch),
ne - 1) (das_kernel_phase_shifts.cu:119-154).  For pitch > width (the reference's own
check) the nearest element outside lies (pitch - width/2)/L beyond u = 1 and the
outermost inside width/2/L within, so both rules agree; this checks it in FP32 on
random geometries, down to a width of 1e-3 pitch."""
import numpy as np


def _index_rule(ne, M, pitch, width, x, h):
    e = np.arange(ne)
    c = (e - M) * pitch
    ilb = max(int(np.ceil(M + (x - h) / pitch)), 0)
    iub = min(int(np.floor(M + (x + h) / pitch)), ne - 1)
    emid = int(np.searchsorted(c, x, side="left"))
    left = e < emid
    return np.where(left, e >= ilb, e <= iub), c, ilb, iub, left


def _u_rule(ne, c, pitch, width, x, ilb, iub, left):
    f32 = np.float32
    il = f32(1e30)
    ir = f32(1e30)
    if ilb < ne:
        L = f32(x - (c[ilb] - width / 2))
        if L > 0:
            il = f32(1.0) / L
    if iub >= 0:
        L = f32((c[iub] + width / 2) - x)
        if L > 0:
            ir = f32(1.0) / L
    d = np.abs(c - x).astype(f32)
    dl = np.where(left, d, f32(0.0)).astype(f32)
    dr = np.where(left, f32(0.0), d).astype(f32)
    u = (dl * il + dr * ir).astype(f32)
    return u < 1, u


def test_membership_by_window_argument_matches_index_rule():
    rng = np.random.default_rng(5)
    worst = np.inf
    for _ in range(4000):
        ne = int(rng.integers(2, 257))
        pitch = float(rng.uniform(0.1e-3, 0.5e-3))
        width = pitch * float(10 ** rng.uniform(-3, np.log10(0.99)))
        M = (ne - 1) / 2.0
        extent = ne * pitch
        x = float(rng.uniform(-0.7, 0.7) * extent)
        h = float(rng.uniform(0.0, 60e-3)) if rng.random() < 0.9 else float(rng.uniform(0, pitch))
        want, c, ilb, iub, left = _index_rule(ne, M, pitch, width, x, h)
        got, u = _u_rule(ne, c, pitch, width, x, ilb, iub, left)
        assert np.array_equal(got, want), (ne, pitch, width, x, h)
        # every member lies in [i_lb, i_ub]: the adjoint skips the warps whose elements
        # miss that range for all of their voxels (a side without aperture, i_lb = ne or
        # i_ub = -1, leaves the voxel beyond the array's end, with no element on the other
        # side of it either)
        e = np.arange(ne)
        assert not np.any(want & ((e < ilb) | (e > iub))), (ne, pitch, width, x, h)
        finite = np.isfinite(u) & (u < 1e20)
        if finite.any():
            worst = min(worst, float(np.min(np.abs(u[finite] - 1.0))))
    # the closest element to the boundary stays well clear of FP32 rounding
    assert worst > 1e-6
