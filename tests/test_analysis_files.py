"""The file-driven estimators (stats.statistical_analysis_of_pimc / jackknife_analysis_of_pimc and
the postprocessing helpers they use) against the *_thermo files the reference itself wrote from the
same data set (tests/golden/make_golden.py: stats.py:148-179, 219-265, 336-377;
postprocessing.py:48-58, 118-144, 294-340).

Host logic only: no device is touched."""
import glob
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from pibronic_gb300 import file_structure, postprocessing, stats

RUNS = [("stats", "basic"), ("stats", "alpha"), ("jk", "basic"), ("jk", "alpha")]


@pytest.fixture(scope="module")
def ref():
    with np.load(os.path.join(GOLDEN, "reference_analysis_files.npz")) as d:
        return {k: d[k] for k in d.files}


def _data_set(ref, root):
    FS = file_structure.FileStructure(str(root), 0, 0)
    with open(FS.path_vib_model, "w") as fh:
        fh.write(str(ref["vib_json"]))
    with open(FS.path_rho_model, "w") as fh:
        fh.write(str(ref["rho_json"]))
    with open(FS.path_analytic_rho, "w") as fh:
        fh.write(str(ref["analytic_json"]))
    for k, v in ref.items():
        if k.startswith("result/"):
            with open(os.path.join(FS.path_rho_results, k[len("result/"):]), "wb") as fh:
                fh.write(v.tobytes())
    return FS


def _thermo_of(ref, tag, method):
    pre = f"thermo/{tag}_{method}/"
    return {k[len(pre):]: json.loads(str(v)) for k, v in ref.items() if k.startswith(pre)}


@pytest.mark.parametrize("tag,method", RUNS)
def test_thermo_files_match_the_reference(ref, tag, method, tmp_path):
    FS = _data_set(ref, tmp_path)
    driver = stats.statistical_analysis_of_pimc if tag == "stats" else stats.jackknife_analysis_of_pimc
    written = driver(FS, method=method)
    expect = _thermo_of(ref, tag, method)
    found = sorted(glob.glob(os.path.join(FS.path_rho_results, "*_thermo")))
    assert sorted(map(os.path.basename, found)) == sorted(expect) == sorted(map(os.path.basename, written))
    for path in found:
        with open(path) as fh:
            mine = json.loads(fh.read())
        want = expect[os.path.basename(path)]
        assert list(mine) == list(want)
        for k, v in want.items():
            if isinstance(v, str):
                assert mine[k] == v, k
            else:
                # the merge adds the jobs' samples in another order than the reference's set order
                assert np.isclose(mine[k], v, rtol=1e-10, atol=1e-300), (path, k, mine[k], v)


def test_model_hashes_match_the_reference(ref, tmp_path):
    FS = _data_set(ref, tmp_path)
    FS.generate_model_hashes()
    stored = json.loads(str(ref["analytic_json"]))
    assert FS.hash_vib == stored["hash_vib"] and FS.hash_rho == stored["hash_rho"]
    with np.load(os.path.join(FS.path_rho_results, "P12_T300.00_J0_data_points.npz")) as d:
        assert str(d["hash_vib"]) == FS.hash_vib and str(d["hash_rho"]) == FS.hash_rho


def test_result_file_lists_and_parameters(ref, tmp_path):
    FS = _data_set(ref, tmp_path)
    files = postprocessing.retrive_pimc_file_list(FS)
    assert len(files) == sum(k.startswith("result/") for k in ref)
    assert postprocessing.extract_bead_paramater_list(files) == [8, 12]
    assert postprocessing.extract_temperature_paramater_list(files) == [250.0, 300.0]
    jobs = sorted(postprocessing.extract_job_value_from_pimc_file_path(f) for f in files)
    assert jobs == [0, 0, 0, 0, 1, 1]
    FS.generate_model_hashes()
    assert sorted(postprocessing.prune_results_using_hashes(FS, files)) == sorted(files)
    FS.hash_rho = "0" * 128
    assert postprocessing.prune_results_using_hashes(FS, files) == []
    with pytest.raises(Exception):
        postprocessing.prune_results_using_hashes(FS, [FS.path_vib_model])


def test_thermo_file_name_parsing(ref, tmp_path):
    FS = _data_set(ref, tmp_path)
    stats.jackknife_analysis_of_pimc(FS, method="basic")
    paths = postprocessing.retrive_jackknife_file_list(FS)
    got = sorted((postprocessing.extract_bead_value_from_thermo_file_path(p),
                  postprocessing.extract_temperature_value_from_thermo_file_path(p),
                  postprocessing.extract_sample_value_from_thermo_file_path(p)) for p in paths)
    assert got == [(8, 250.0, 30), (8, 300.0, 20), (12, 250.0, 20), (12, 300.0, 80)]
    assert sorted(postprocessing.prune_results_using_hashes(FS, paths)) == sorted(paths)


def test_bad_method_and_location_are_rejected(ref, tmp_path):
    FS = _data_set(ref, tmp_path)
    with pytest.raises(Exception):
        stats.statistical_analysis_of_pimc(FS, method="gamma")
    with pytest.raises(AssertionError):
        stats.jackknife_analysis_of_pimc(FS, method="basic", location="server")
    with pytest.raises(Exception):
        stats.jackknife_analysis_of_pimc(FS, method="basic", location="moon")


def test_analytic_file_with_other_hashes_is_rejected(ref, tmp_path):
    FS = _data_set(ref, tmp_path)
    stored = json.loads(str(ref["analytic_json"]))
    stored["hash_vib"] = "f" * 128
    with open(FS.path_analytic_rho, "w") as fh:
        fh.write(json.dumps(stored))
    with pytest.raises(AssertionError):
        stats.statistical_analysis_of_pimc(FS, method="basic")
