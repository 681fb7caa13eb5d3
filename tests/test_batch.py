"""Manifest runner (hybrid-bicg_gb300/run_manifest.py): how a manifest expands
into runs — matrices from generators and Matrix Market files, shift and
right-hand-side specifications, one run per seed (the reference's seed sweep,
src/main_seed_diff.c:113-155).  No GPU needed."""
import importlib.util

import numpy as np
import pytest
from conftest import ROOT


@pytest.fixture(scope="module")
def rm():
    spec = importlib.util.spec_from_file_location("run_manifest", ROOT / "hybrid-bicg_gb300" / "run_manifest.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_expand_generators_shifts_rhs_and_seeds(rm, pkg, tmp_path):
    np.save(tmp_path / "b.npy", np.arange(64, dtype=np.float64))
    man = {"families": [
        {"name": "a", "matrix": {"generator": "stencil_cd3d", "args": [4]}, "shifts": {"linspace": [0.0, 0.15, 16]},
         "seeds": [0, 5, 15]},
        {"name": "b", "matrix": {"generator": "stencil_cd3d", "args": [4]}, "shifts": [0.1, 0.2], "rhs": "b.npy"},
        {"name": "c", "matrix": {"generator": "stencil_cd2d", "args": [6]}, "shifts": {"geomspace": [1e-4, 1, 5]},
         "rhs": {"normal": 3}},
    ]}
    runs = rm.expand(man, tmp_path, pkg)
    assert [(r.name, r.seed) for r in runs] == [("a", 0), ("a", 5), ("a", 15), ("b", 0), ("c", 0)]
    assert runs[0].a is runs[3].a  # one matrix object for one spec
    assert np.allclose(runs[0].sigma, 0.01 * np.arange(16))
    assert np.allclose(runs[0].b, 1.0 / np.sqrt(64))  # the reference's b
    assert np.array_equal(runs[3].b, np.arange(64.0))
    assert np.allclose(runs[4].sigma, np.geomspace(1e-4, 1, 5))
    assert np.array_equal(runs[4].b, np.random.default_rng(3).standard_normal(36))


def test_expand_matrix_market_file_in_reference_row_order(rm, pkg, tmp_path):
    a = pkg.workloads.stencil_cd3d(5, 4, 3)
    pkg.workloads.write_matrix_market(str(tmp_path / "a.mtx"), a)
    runs = rm.expand({"families": [{"matrix": "a.mtx", "shifts": [0.0]}]}, tmp_path, pkg)
    got = runs[0].a
    assert np.array_equal(got.ptr, a.ptr) and np.array_equal(got.col, a.col) and np.array_equal(got.val, a.val)


@pytest.mark.parametrize("fam,what", [
    ({"matrix": {"generator": "stencil_cd3d", "args": [3]}, "shifts": [0.0, 0.1], "seeds": [2]}, "seed"),
    ({"matrix": {"generator": "nope"}, "shifts": [0.0]}, "generator"),
    ({"matrix": {"generator": "stencil_cd3d", "args": [3]}, "shifts": {"range": 3}}, "shifts"),
])
def test_expand_rejects_bad_entries(rm, pkg, tmp_path, fam, what):
    with pytest.raises(ValueError, match=what):
        rm.expand({"families": [fam]}, tmp_path, pkg)


def test_family_struct_matches_header(pkg):
    """hbicg_family's field order and C layout (include/hbicg.h)."""
    F = pkg.Family
    assert [f[0] for f in F._fields_][:10] == ["n", "nnz", "ptr", "col", "val", "b", "sigma", "m", "seed", "autotune"]
    assert F.x.offset == 64 and F.status.offset == 88 and F.solve_ms.offset == 112 and F.max_true_residual.offset == 128
