"""Output files of MonteCarlo(outpath=...) and the drivers (monte_carlo.jl:95-116,
:186-188, :353-364, :387-391) in hdf5.jl's layout, on the GPU path."""
import importlib
import os

import numpy as np
import pytest

from test_hdf5 import _sorted_cell, validate

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def h5(m):
    return importlib.import_module(m.__name__ + ".hdf5")


def _pt(m, out, seed=4, **kw):
    uc = m.examples.triangular_afm(h=0.3)
    lat = m.Lattice((6, 6), uc, 1.0)
    lat.spins[:] = m.examples.random_spins(lat.size, seed=seed)
    mc = m.MonteCarlo([0.2, 0.4, 0.9], lat, {"overrelaxation_rate": 5}, precision="fp64", seed=seed,
                      outpath=out, **kw)
    p = mc.parameters
    p.t_thermalization, p.t_measurement, p.report_interval, p.checkpoint_rate = 10, 30, 15, 10
    p.probe_rate, p.swap_rate = 5, 5
    return lat, mc


def test_parallel_tempering_writes_the_reference_files(m, h5, tmp_path, capsys):
    out = str(tmp_path / "run") + "/"
    lat, mc = _pt(m, out, inparams={"J": 1.0, "model": "triangular"})
    assert mc.outpath == [out + f"configuration_{r}.h5" for r in range(3)]
    assert "Creating new file configuration_2.h5 for output on rank 2" in capsys.readouterr().out
    res = m.parallel_tempering(mc, saveIC=(0, 2), verbose=False)
    names = sorted(os.listdir(out))
    assert names == ["IC_0", "IC_2", "configuration.h5.params", "configuration_0.h5", "configuration_1.h5",
                     "configuration_2.h5"]
    assert sorted(os.listdir(out + "IC_0")) == ["IC_0.h5", "IC_1.h5", "IC_2.h5"]
    for fn in names[2:]:
        validate(open(out + fn, "rb").read())
    with h5.h5open(out + "configuration.h5.params") as f:
        L = h5.read_lattice(f)
        assert f.attrs["J"] == 1.0 and f.attrs["model"] == "triangular" and f.attrs["checkpoint_rate"] == 0
    want = m.Lattice((6, 6), _sorted_cell(m, lat.unit_cell), 1.0)  # terms come back in key-name order
    for k, v in want.tables().items():
        assert np.array_equal(L.tables()[k], v)
    for r in range(3):
        with h5.h5open(mc.outpath[r]) as f:
            assert f.attrs["T"] == mc.temperatures[r]
            assert f.attrs["paramsfile"] == out + "configuration.h5.params"
            assert np.array_equal(f["spins"].read(), mc.spins(r).T)  # the final spins
            s = res["summary"][r]
            g = f["observables"]
            assert float(g["energy"].read()) == s["energy"]
            assert float(g["specific_heat"].read()) == s["specific_heat"]
            assert float(g["specific_heat_err"].read()) == pytest.approx(abs(s["specific_heat_err"] / s["specific_heat"]))
            assert float(g["susceptibility_err"].read()) == pytest.approx(
                abs(s["susceptibility_err"] / s["susceptibility"]))
    for r in (0, 2):
        for ts in range(3):
            with h5.h5open(out + f"IC_{r}/IC_{ts}.h5") as f:
                assert np.array_equal(f["spins"].read(), mc.initial_configurations[r][ts].T)
                assert f.attrs["T"] == mc.temperatures[r]
    # an existing params file is kept, as the reference keeps it (monte_carlo.jl:102)
    before = open(out + "configuration.h5.params", "rb").read()
    _pt(m, out, seed=5)
    assert open(out + "configuration.h5.params", "rb").read() == before


def test_checkpoints_and_file_output_do_not_change_the_chains(m, h5, tmp_path):
    """The per-checkpoint downloads and the per-temperature annealing calls
    that file output needs leave every chain as it is without files."""
    _, a = _pt(m, "")
    _, b = _pt(m, str(tmp_path / "pt") + "/")
    ra = m.parallel_tempering(a, verbose=False)
    rb = m.parallel_tempering(b, verbose=False)
    assert np.array_equal(ra["energy"], rb["energy"])
    for r in range(3):
        assert np.array_equal(a.spins(r), b.spins(r))
    uc = m.examples.honeycomb_kitaev(K=-1, J=0.1, G=0.05)
    lat = m.Lattice((6, 6), uc, 1.0)
    lat.spins[:] = m.examples.random_spins(lat.size, seed=3)
    runs = []
    for out in ("", str(tmp_path / "sa") + "/"):
        mc = m.MonteCarlo(1e-2, lat, {"t_thermalization": 20, "overrelaxation_rate": 4}, precision="fp64", seed=9,
                          outpath=out)
        acc = m.simulated_annealing(mc, lambda t: 0.6 ** t, 1.0, verbose=False)
        runs.append((acc, mc.spins(0), mc))
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])
    with h5.h5open(runs[1][2].outpath) as f:  # the last checkpoint holds the final spins
        assert np.array_equal(f["spins"].read(), runs[1][1].T)


def test_structure_factor_of_stored_configurations(m, h5, orc, tmp_path):
    """runEqualTimeStructureFactor! and compute_equal_time_structure_factor
    (spin_correlations.jl:48-145) over IC files: batched device launches, the
    oracle's correlations per file, skip / override, the rank split, the mean."""
    uc = m.examples.honeycomb_kitaev(K=-1, J=0.1)
    lat = m.Lattice((4, 5), uc, 1.0)
    ks = m.get_allowed_wavevectors(uc, (4, 5))[:, ::2]
    path = str(tmp_path / "IC_0") + "/"
    os.mkdir(path)
    spins = [m.examples.random_spins(lat.size, seed=i) for i in range(7)]
    for i, s in enumerate(spins):
        with h5.h5open(path + f"IC_{i}.h5", "w") as f:
            f.attrs["T"] = 0.5
            f.attrs["paramsfile"] = "configuration.h5.params"
            f["spins"] = s.T
    # two "ranks": 4 + 3 files, in batches of 3 and 2 configurations
    assert m.runEqualTimeStructureFactor(path, lat, ks, rank=0, world=2, batch=3, verbose=False) == [0, 1, 2, 3]
    assert m.runEqualTimeStructureFactor(path, lat, ks, rank=1, world=2, batch=2, verbose=False) == [4, 5, 6]
    refs = []
    for i, s in enumerate(spins):
        with h5.h5open(path + f"IC_{i}.h5") as f:
            got = f["spin_correlations/SSF"].read().T
            assert np.array_equal(f["spin_correlations/SSF_momentum"].read(), ks.T)
        refs.append(orc.structure_factor(s, lat.site_positions, ks))
        assert np.abs(got - refs[-1]).max() <= 1e-10 * lat.size
    assert m.runEqualTimeStructureFactor(path, lat, ks, verbose=False) == []  # all present: skipped
    assert m.runEqualTimeStructureFactor(path, lat, ks, override=True, batch=64, verbose=False) == list(range(7))
    dest = str(tmp_path / "configuration_0.h5")
    with h5.h5open(dest, "w") as f:
        f["spins"] = spins[0].T
    mean = m.compute_equal_time_structure_factor(path, dest, verbose=False)
    assert np.abs(mean - np.mean(refs, axis=0)).max() <= 1e-10 * lat.size
    with h5.h5open(dest) as f:
        assert np.array_equal(f["spin_correlations/SSF"].read(), mean.T)
        assert np.array_equal(f["spin_correlations/SSF_momentum"].read(), ks.T)
    validate(open(dest, "rb").read())
