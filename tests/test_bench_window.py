"""Host logic of the bench's timed window and roofline units (bench.py): where the window starts,
and the node counts the E/B and gather byte figures use, on small made-up bunches."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_window_starts_at_ninety_percent_or_early_enough_for_the_legs():
    # the bench job: 1905 steps; K steps timed after W warm-up, then K instrumented, the e2e leg
    # re-runs K from the window's start, and the one-thread oracle leg takes up to 3 more
    assert bench.window_start(1905, 3, 10) == 1714
    assert bench.window_start(1905, 3, 100) == 1905 - 3 - 300 - 3
    assert bench.window_start(100, 3, 10) == 64
    assert bench.window_start(20, 3, 10) == 3  # never before the graph-capture warm-up


def _meta(n0=6, n1=5, nz=7):
    return {"xmin": -1.0, "ymin": -2.0, "zmin": 0.5, "dx": 0.5, "dy": 1.0, "dz": 0.25,
            "N0": n0, "N1": n1, "np": nz}


def _parts(cells, meta, rng):
    """Particle records whose positions lie inside the given (i, j, k) cells."""
    out = np.zeros((len(cells), 11))
    for r, (i, j, k) in enumerate(cells):
        f = rng.uniform(0.05, 0.95, 3)
        out[r, 1] = meta["xmin"] + (i + f[0]) * meta["dx"]
        out[r, 2] = meta["ymin"] + (j + f[1]) * meta["dy"]
        out[r, 3] = meta["zmin"] + (k + f[2]) * meta["dz"]
    return out


def test_touched_nodes_counts_the_corners_of_occupied_cells_once():
    rng = np.random.default_rng(3)
    m = _meta()
    # two particles in one cell, one in the cell next to it along x: 8 + 4 corner nodes
    p = _parts([(1, 1, 1), (1, 1, 1), (2, 1, 1)], m, rng)
    assert bench.touched_nodes(p, m) == 12
    # a cell diagonal to the first shares one corner only
    p = _parts([(1, 1, 1), (2, 2, 2)], m, rng)
    assert bench.touched_nodes(p, m) == 15
    # particles outside the mesh read nothing
    p = _parts([(1, 1, 1)], m, rng)
    p = np.vstack([p, [[0.0, -50.0, 0.0, 0.0] + [0.0] * 7]])
    assert bench.touched_nodes(p, m) == 8


def test_slab_nodes_cover_the_particle_planes_with_their_margins():
    rng = np.random.default_rng(4)
    m = _meta(nz=12)
    p = _parts([(1, 1, 4), (2, 2, 6)], m, rng)
    # planes 4-2 .. 6+3 = 2 .. 9, interior nodes per plane (6-2) x (5-2)
    assert bench.slab_nodes(p, m) == 8 * 4 * 3
    # clipped to the interior planes 1 .. np-2 at the mesh ends
    p = _parts([(1, 1, 0), (1, 1, 10)], m, rng)
    assert bench.slab_nodes(p, m) == 10 * 4 * 3


def test_surrogate_line_rates_and_keys():
    """The surrogate workload's bench line: screened designs/h = 3600 / (inference + fallback x
    full solve), the full solver's designs/h, the row of the chosen threshold."""
    out = {"solve_s_per_design": 0.032, "infer_s_per_design": 3e-5, "train_steps": 6000, "train_s": 25.0,
           "median_err": 0.022, "p90_err": 0.066, "baseline_median_err": 0.9,
           "screening": [{"threshold": 0.05, "fallback": 0.1, "accepted_median_err": 0.021,
                          "accepted_p90_err": 0.06, "speedup": 9.9},
                         {"threshold": 0.1, "fallback": 0.001, "accepted_median_err": 0.022,
                          "accepted_p90_err": 0.066, "speedup": 500.0}]}
    line = bench.surrogate_line(out, 16384, 1024, 0.1, {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                                                         "samples": 0})
    assert line["value"] == 3600.0 / (3e-5 + 0.001 * 0.032)
    assert line["full_solve_designs_per_hour"] == 3600.0 / 0.032
    assert line["held_out_psat_error"]["fallback"] == 0.001 and line["speedup_vs_full_solve"] == 500.0
    assert line["config"]["workload"] == "surrogate-48x48x384" and line["config"]["threshold"] == 0.1
    for k in ("metric", "unit", "n_gpus", "higher_is_better", "dtype", "clocks"):
        assert k in line
