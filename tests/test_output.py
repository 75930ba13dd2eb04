"""Field output (PRTSCR, 4_plot.f90:547-615) on CPU: the oracle's record
read back as a Fortran unformatted sequential file (gfortran framing) and
checked array by array against numpy on the oracle's own fields."""
import numpy as np
import pytest

from helpers import oracle_for
from suli_gb300 import cases


def read_fortran_record(path):
    """The single record of a gfortran unformatted sequential file: a 4-byte
    little-endian byte count, the bytes, the same count again."""
    raw = open(path, "rb").read()
    n = int(np.frombuffer(raw[:4], "<i4")[0])
    tail = int(np.frombuffer(raw[4 + n:8 + n], "<i4")[0])
    assert n == tail and len(raw) == n + 8, (n, tail, len(raw))
    return np.frombuffer(raw[4:4 + n], "<f4")


def split_record(rec, p, t_plot):
    """Arrays of the record in Fortran order: x, y, z, u, v, w at the cell
    corners (nx+1, ny+1, nz+1), ls at the cells, obs_ls at the corners, and
    with t_plot = 1 pressure, three vorticity components, nut, ka at the cells."""
    n1 = (p.nx + 1, p.ny + 1, p.nz + 1)
    nc = (p.nx, p.ny, p.nz)
    shapes = [n1] * 6 + [nc, n1] + ([nc] * 6 if t_plot else [])
    out, o = [], 0
    for s in shapes:
        m = int(np.prod(s))
        out.append(rec[o:o + m].reshape(s, order="F"))
        o += m
    assert o == rec.size
    return out


def expected(o, p, t_plot):
    u, v, w = o.field("U"), o.field("V"), o.field("W")     # u(0:nx+2, 0:ny+1, 0:nz+1) etc.
    nx, ny, nz = p.nx, p.ny, p.nz
    I, J, K = slice(1, nx + 2), slice(1, ny + 2), slice(1, nz + 2)
    Im, Jm, Km = slice(0, nx + 1), slice(0, ny + 1), slice(0, nz + 1)
    ua = (u[I, J, K] + u[I, Jm, K] + u[I, J, Km] + u[I, Jm, Km]) * 0.25
    va = (v[I, J, K] + v[Im, J, K] + v[I, J, Km] + v[Im, J, Km]) * 0.25
    wa = (w[I, J, K] + w[I, Jm, K] + w[Im, J, K] + w[Im, Jm, K]) * 0.25
    x = np.cumsum(np.r_[-p.dx, np.full(nx + 1, p.dx)])[1:]
    y = np.cumsum(np.r_[-p.dy, np.full(ny + 1, p.dy)])[1:]
    z = np.cumsum(np.r_[-p.dz, np.full(nz + 1, p.dz)])[1:]
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    obs = o.field("OBS_LS") if p.obst_t else np.zeros(X.shape)
    arrs = [X, Y, Z, ua, va, wa, o.field("LS"), obs]
    if t_plot:
        c = slice(1, nx + 1), slice(1, ny + 1), slice(1, nz + 1)
        pr = o.field("PRD0") + o.field("PRD1")          # prd0 = 0 unless the IPA ran (4_plot.f90:573)
        i, j, k = c
        ip, jp, kp = slice(2, nx + 2), slice(2, ny + 2), slice(2, nz + 2)
        dudy = (u[i, jp, k] - u[i, j, k]) / p.dy
        dudz = (u[i, j, kp] - u[i, j, k]) / p.dz
        dvdx = (v[ip, j, k] - v[i, j, k]) / p.dx
        dvdz = (v[i, j, kp] - v[i, j, k]) / p.dz
        dwdx = (w[ip, j, k] - w[i, j, k]) / p.dx
        dwdy = (w[i, jp, k] - w[i, j, k]) / p.dy
        arrs += [pr[c] - pr[nx, 1, nz], dwdy - dvdz, dudz - dwdx, dvdx - dudy, o.field("NUT"),
                 o.field("KA")[c]]
    return arrs


@pytest.mark.parametrize("t_plot", [0, 1])
@pytest.mark.parametrize("kind", ["dam_break", "channel_ibm", "k_les", "ipa"])
def test_oracle_prtscr_record(tmp_path, kind, t_plot):
    if kind == "dam_break":
        case = cases.dam_break(12, 8, 6)
    elif kind == "k_les":
        case = cases.k_channel(16, 6, 10, m_turb=2)
    elif kind == "ipa":
        case = cases.ipa_tank(12, 6, 10)
    else:
        case = cases.open_channel(24, 8, 8, dt=2e-3, radius=0.25, periodic=True)
    o = oracle_for(case, warm_steps=1)
    path = tmp_path / "campos_00010"
    o.prtscr_write(path, t_plot)
    got = split_record(read_fortran_record(path), case.params, t_plot)
    want = expected(o, case.params, t_plot)
    for n, (a, b) in enumerate(zip(got, want)):
        b32 = np.asarray(b, dtype=np.float64).astype(np.float32)
        # the oracle rounds each FP64 value once to float32, as real(x, 4) does;
        # numpy's vectorised sums may differ from the loop in the last FP64 bit
        assert np.allclose(a, b32, rtol=2e-7, atol=1e-7 * max(1.0, float(np.abs(b32).max()))), n
    if kind == "channel_ibm":
        assert np.abs(got[7]).max() > 0          # the obstacle's corner level set is written
