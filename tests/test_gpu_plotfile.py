"""Native plotfile writer (hx_write_plotfile_f64): the level planes of every
box come back bit for bit through an independent parse of the files; the
header carries the reference's variable names, time, extents and steps.

Parity with amrex::WriteMultiLevelPlotfile itself is not pinned (AMReX is not
available here); the layout is AMReX's documented HyperCLaw-V1.1 one."""
import numpy as np
import pytest
import torch

from hydroexa_gb300 import capi
from hydroexa_gb300.plotfile import VARIABLES, PlotBox, PlotLevel, read_plotfile, write_plotfile

pytestmark = pytest.mark.gpu


def _boxes(rng, dev, spans):
    out = []
    for (x0, y0, x1, y1) in spans:
        ny, nx = y1 - y0 + 1, x1 - x0 + 1
        S = torch.from_numpy(rng.uniform(-1, 3, size=(3, ny, nx))).to(dev)
        T = torch.from_numpy(rng.uniform(-2, 1, size=(2, ny, nx))).to(dev)
        out.append(PlotBox(S, T, (x0, y0)))
    return out


def test_single_level_round_trip(cuda, tmp_path):
    rng = np.random.default_rng(3)
    spans = [(0, 0, 31, 23), (32, 0, 63, 23), (0, 24, 40, 47), (41, 24, 63, 47)]
    boxes = _boxes(rng, cuda, spans)
    lev = PlotLevel(boxes, (0, 0), (63, 47), 1.0 / 64, 1.0 / 48, istep=17)
    d = write_plotfile(str(tmp_path / "plt"), 17, 0.125, [lev])
    assert d.name == "plt00017"
    pf = read_plotfile(d)
    assert pf["version"] == "HyperCLaw-V1.1" and pf["variables"] == list(VARIABLES) and pf["dim"] == 2
    assert pf["time"] == 0.125 and pf["steps"] == [17] and pf["domains"] == [(0, 0, 63, 47)]
    assert pf["prob_lo"] == [0.0, 0.0] and pf["prob_hi"] == [1.0, 1.0]
    assert pf["cell_size"] == [[1.0 / 64, 1.0 / 48]] and pf["coord_sys"] == 0
    L = pf["levels"][0]
    assert len(L["boxes"]) == 4
    for (lo, hi, arr), b, (x0, y0, x1, y1) in zip(L["boxes"], boxes, spans):
        assert lo == (x0, y0) and hi == (x1, y1)
        want = torch.cat([b.state, b.terrain]).cpu().numpy()
        assert np.array_equal(arr, want)
    # physical extents of each box, and the per-box minima / maxima of the FabArray header
    assert L["extents"][1] == [[0.5, 1.0], [0.0, 0.5]]
    mins = [ln for ln in L["cell_h"] if ln.count(",") == 5 and not ln.startswith("4,")]
    assert len(mins) == 8
    first = [float(x) for x in mins[0].rstrip(",").split(",")]
    want0 = torch.cat([boxes[0].state, boxes[0].terrain]).cpu().numpy()
    assert first == [float(want0[c].min()) for c in range(5)]


def test_two_levels(cuda, tmp_path):
    rng = np.random.default_rng(5)
    coarse = PlotLevel(_boxes(rng, cuda, [(0, 0, 15, 11)]), (0, 0), (15, 11), 1.0 / 16, 1.0 / 12, 2, 4)
    fine = PlotLevel(_boxes(rng, cuda, [(4, 4, 11, 9), (12, 4, 19, 9)]), (0, 0), (31, 23), 1.0 / 32, 1.0 / 24, 2, 8)
    d = write_plotfile(str(tmp_path / "plt"), 8, 2.5, [coarse, fine])
    pf = read_plotfile(d)
    assert pf["ref_ratio"] == [2] and pf["steps"] == [4, 8] and pf["domains"] == [(0, 0, 15, 11), (0, 0, 31, 23)]
    assert [len(L["boxes"]) for L in pf["levels"]] == [1, 2]
    for L, lev in zip(pf["levels"], (coarse, fine)):
        for (_, _, arr), b in zip(L["boxes"], lev.boxes):
            assert np.array_equal(arr, torch.cat([b.state, b.terrain]).cpu().numpy())


def test_box_outside_domain_is_rejected(cuda, tmp_path):
    rng = np.random.default_rng(7)
    lev = PlotLevel(_boxes(rng, cuda, [(0, 0, 15, 11)]), (0, 0), (14, 11), 0.1, 0.1)
    with pytest.raises(capi.HxError):
        write_plotfile(str(tmp_path / "plt"), 0, 0.0, [lev])
