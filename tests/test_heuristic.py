"""Single-sample heuristic (triangle_setup.comp:826-871, single_sample_heuristic.comp)
in the oracle: flat primitives of a super-sampled pass are demoted to
single-sampled rasterisation (SNAP_RASTER) unless a 3D primitive shares one of
their vertices at a depth the 3D geometry uses; those inside the 3D depth range
go back to per-sample attributes (SNAP_ATTRIBUTE cleared).  Flat lines are
demoted only when the instance has no 3D primitive."""
import numpy as np
import pytest

import gsgen
import pgs
import pgs_oracle

SA, SR = 1 << 26, 1 << 25


def decisions(zpsm, ss=4):
    f = gsgen.frame_flat_ui(zpsm=zpsm, super_sampling=ss)
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be, super_sampling=ss)
    gs.gif_transfer(0, f.data)
    gs.flush()
    st = be.state_log()
    gs.close()
    be.close()
    # Categories in submission order (gsgen.frame_flat_ui).
    nq, nl = 100, 64
    nm = len(st) - 4 * nq - nl - nq - nl
    names = [("mesh", nm), ("shared", nq), ("mesh_depth", nq), ("unused_depth", nq), ("ui", nq),
             ("lines", nl), ("flat_only", nq), ("flat_only_lines", nl)]
    out, o = {}, 0
    for name, n in names:
        out[name] = st[o:o + n]
        o += n
    assert o == len(st)
    return out


@pytest.mark.parametrize("zpsm", [gsgen.PSMZ16, gsgen.PSMZ24, gsgen.PSMZ32])
def test_heuristic_decisions(zpsm):
    d = decisions(zpsm)
    frac = lambda s, bit: float(np.mean((s & bit) != 0))
    # 3D geometry is never snapped.
    assert frac(d["mesh"], SA) == 0 and frac(d["mesh"], SR) == 0
    # Sharing a vertex with the mesh at a mesh depth: not demoted, and within
    # the 3D depth range so per-sample attributes come back.
    assert frac(d["shared"], SR) == 0
    assert frac(d["shared"], SA) <= 0.02
    # UI in front of the mesh: always demoted.
    assert frac(d["ui"], SR) == 1 and frac(d["ui"], SA) == 1
    # Flat triangles at depths without a shared vertex: mostly demoted (the
    # exceptions share their depth value with a "shared" triangle).
    assert frac(d["mesh_depth"], SR) > 0.6
    assert frac(d["unused_depth"], SR) > 0.9
    # Lines keep per-sample rasterisation next to 3D geometry ...
    assert frac(d["lines"], SR) == 0 and frac(d["lines"], SA) == 0
    # ... and are demoted in an instance with no 3D primitive.
    assert frac(d["flat_only_lines"], SR) == 1
    assert frac(d["flat_only"], SR) == 1


def test_heuristic_inactive_without_super_sampling():
    f = gsgen.frame_flat_ui(super_sampling=1)
    be = pgs_oracle.OracleBackend()
    gs = pgs.GSInterface(be, super_sampling=1)
    gs.gif_transfer(0, f.data)
    gs.flush()
    st = be.state_log()
    gs.close()
    be.close()
    assert not np.any(st & (SA | SR))
