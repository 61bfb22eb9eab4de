"""GPU: the learned-proposal data path and the device alpha estimator against the reference.

* block_compute_gR_from_raw_samples and block_compute_rhoR_from_input_samples (pimc.py:1273-1338)
  run on the FP64 stage kernels and are held to the reference's own run of the same case
  (tests/golden/reference_runs.npz, "ml/"): the same uniform R (numpy's generator, consumed as the
  reference's preprocess consumes it), g(R) and rho(R) to a relative 1e-9, and the training files
  (pimc.py:1250-1270) with the reference's names, keys, dtypes, R values bit for bit and g(R)
  values to a relative 1e-9.
* stats.device_alpha_estimates (the alpha estimator and its jackknife on the device reduction
  kernels) against the host alpha_jackknife_analysis (stats.py:302-333, jackknife.py:14-57) on
  the result files of the reference-written analysis data set, and the basic device estimates
  against basic_jackknife_analysis (stats.py:271-299) on the same files.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, case_of

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ML = dict(A=2, N=3, P=8, T=300.0, X=30, B=15, rng_seed=2024)    # make_golden.py ML_CASE


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pibronic_gb300 import build, _native
    _native.load(build.build())


def _ml_data(runs, tmp_path):
    from pibronic_gb300 import pimc
    from pibronic_gb300.file_structure import FileStructure
    c = case_of(runs, "ml")
    FS = FileStructure(str(tmp_path), 0, 0)
    with open(FS.path_vib_model, "w") as fh:
        fh.write(str(c["vib_json"]))
    with open(FS.path_rho_model, "w") as fh:
        fh.write(str(c["rho_json"]))
    FS.generate_model_hashes()
    data = pimc.BoxData.from_FileStructure(FS)
    data.hash_vib, data.hash_rho = FS.hash_vib, FS.hash_rho
    data.samples, data.beads, data.temperature = ML["X"], ML["P"], ML["T"]
    data.block_size = ML["B"]
    data.blocks = data.samples // data.block_size
    data.preprocess()
    return c, FS, data


def test_g_of_R_and_training_files_match_the_reference(runs, tmp_path):
    from pibronic_gb300 import pimc
    c, FS, data = _ml_data(runs, tmp_path)
    # the reference's preprocess draws the X sample sources from numpy's global generator
    # (pimc.py:386) before block_compute_gR_from_raw_samples draws R (pimc.py:602-611)
    np.random.seed(ML["rng_seed"])
    np.random.choice(range(data.rho.states), size=data.samples, p=data.rho.state_weight)
    result = pimc.BoxResult(data=data)
    result.id_job = 0
    result.path_root = FS.path_vib_results
    pimc.block_compute_gR_from_raw_samples(data, result)
    with np.load(os.path.join(GOLDEN, "reference_training_files.npz")) as f:
        ref = {k: f[k] for k in f.files}
    names = sorted(k for k in ref if k.endswith(".npz"))
    assert names == sorted(n for n in os.listdir(FS.path_vib_results) if "_training_data_" in n)
    for name in names:
        path = os.path.join(str(tmp_path), "ref_" + name)
        with open(path, "wb") as fh:
            fh.write(ref[name].tobytes())
        with np.load(path) as want, np.load(os.path.join(FS.path_vib_results, name)) as got:
            assert sorted(got.files) == sorted(want.files), name
            for k in want.files:
                assert got[k].dtype == want[k].dtype and got[k].shape == want[k].shape, (name, k)
                if k == "g":
                    assert np.allclose(got[k], want[k], rtol=1e-9, atol=0), name
                else:
                    assert np.array_equal(got[k], want[k]), (name, k)
    with np.load(os.path.join(FS.path_vib_results, next(n for n in names if n.endswith("_input.npz")))) as d:
        R = d["input_R_values"]
    assert np.array_equal(R, c["R"])
    assert np.allclose(np.asarray(result.scaled_g), c["g"], rtol=1e-9, atol=0)


def test_rho_of_R_matches_the_reference(runs, tmp_path):
    from pibronic_gb300 import pimc
    c, FS, data = _ml_data(runs, tmp_path)
    res = pimc.BoxResult(data=data)
    pimc.block_compute_rhoR_from_input_samples(data, res, c["R"])
    assert np.allclose(np.asarray(res.scaled_rho), c["rho"], rtol=1e-9, atol=0)


@pytest.fixture(scope="module")
def analysis():
    with np.load(os.path.join(GOLDEN, "reference_analysis_files.npz")) as d:
        return {k: d[k] for k in d.files}


def _data_set(ref, root):
    from pibronic_gb300 import file_structure
    FS = file_structure.FileStructure(str(root), 0, 0)
    for path, key in ((FS.path_vib_model, "vib_json"), (FS.path_rho_model, "rho_json"),
                      (FS.path_analytic_rho, "analytic_json")):
        with open(path, "w") as fh:
            fh.write(str(ref[key]))
    for k, v in ref.items():
        if k.startswith("result/"):
            with open(os.path.join(FS.path_rho_results, k[len("result/"):]), "wb") as fh:
                fh.write(v.tobytes())
    return FS


@pytest.mark.parametrize("P,T", [(12, 300.0), (12, 250.0), (8, 300.0)])
def test_device_alpha_and_basic_estimators_match_host(analysis, tmp_path, P, T):
    from pibronic_gb300 import constants, postprocessing, stats
    from pibronic_gb300.pimc import BoxResultPM
    FS = _data_set(analysis, tmp_path)
    res = BoxResultPM()
    postprocessing.load_pimc_data(FS, P, T, res)
    rho_data = {}
    postprocessing.load_analytic_data(FS, T, rho_data)
    db = constants.delta_beta
    arrays = [torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")
              for a in (res.scaled_rho, res.scaled_g, res.scaled_gofr_plus, res.scaled_gofr_minus)]
    for host, dev in (
            (stats.alpha_jackknife_analysis(T, res, rho_data, db),
             stats.device_alpha_estimates(*arrays, T, db, rho_data["alpha_plus"], rho_data["alpha_minus"])),
            (stats.basic_jackknife_analysis(T, res, rho_data, db),
             stats.device_estimates(*arrays, T, db))):
        # the host dicts carry the sampling model's E and Cv (add_harmonic_contribution)
        dev_full = {"Z": dev["Z"], "Z error": dev["Z error"], "E": dev["E"] + rho_data["E"],
                    "Cv": dev["Cv"] + rho_data["Cv"], "jk_E": dev["jk_E"] + rho_data["E"],
                    "jk_E error": dev["jk_E error"], "jk_Cv": dev["jk_Cv"] + rho_data["Cv"],
                    "jk_Cv error": dev["jk_Cv error"]}
        # Cv subtracts two terms ~1e2 x larger than itself, and the jackknife multiplies by X on
        # top: two FP64 summation orders differ there by a few 1e-6 relative (measured up to 9e-6
        # on the jackknife errors), so the energies and heat capacities are held to 1e-3 of their
        # statistical errors, the errors themselves to 1e-4 relative and Z to 1e-6 relative
        sig = {"E": host["jk_E error"], "jk_E": host["jk_E error"], "Cv": host["jk_Cv error"],
               "jk_Cv": host["jk_Cv error"]}
        for k, v in dev_full.items():
            tol = 1e-3 * sig[k] if k in sig else (1e-4 if k.endswith("error") else 1e-6) * abs(host[k])
            assert abs(v - host[k]) <= tol, (k, v, host[k], tol)
    assert json.loads(str(analysis["analytic_json"]))
