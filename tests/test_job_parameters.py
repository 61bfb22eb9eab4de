"""The job scripts' host sequence (server/compute_canada/pimc.py:20-36) up to the block loop,
against the reference's own run of it (tests/golden/make_golden.py): the submitter's serialised
parameters read by BoxDataPM.from_json_string (pimc.py:543-593), preprocess's beta and tau values
(pimc.py:647-738), the model hashes, and the result file path of a job id given as a string.

Host logic only: preprocess runs with its device step (initialize_models, which uploads the
model tables) replaced by a no-op, so the values it sets before that step are checked on the CPU."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from pibronic_gb300 import file_structure, pimc


@pytest.fixture(scope="module")
def ref():
    with np.load(os.path.join(GOLDEN, "reference_job_parameters.npz")) as d:
        return {k: d[k] for k in d.files}


def _data_set(ref, root):
    fields = {k[len("field/"):]: v for k, v in ref.items() if k.startswith("field/")}
    D, R = int(fields["id_data"]), int(fields["id_rho"])
    FS = file_structure.FileStructure(str(root), D, R)
    with open(FS.path_vib_model, "w") as fh:
        fh.write(str(ref["vib_json"]))
    with open(FS.path_rho_model, "w") as fh:
        fh.write(str(ref["rho_json"]))
    return str(ref["json"]).replace("@ROOT@", str(root)), fields


def test_parameters_from_the_submitter_string(ref, tmp_path):
    text, want = _data_set(ref, tmp_path)
    data = pimc.BoxDataPM.from_json_string(text)
    for k in ("samples", "blocks", "states", "beads", "modes", "block_size", "id_data", "id_rho"):
        assert getattr(data, k) == int(want[k]), k
    for k in ("temperature", "beta", "tau", "delta_beta"):
        assert getattr(data, k) == float(want[k]), k
    assert data.hash_vib == str(want["hash_vib"]) and data.hash_rho == str(want["hash_rho"])


@pytest.fixture
def host_only(monkeypatch):
    monkeypatch.setattr(pimc.BoxData, "initialize_models", lambda self: None)


def test_preprocess_and_result_path_like_the_job_script(ref, tmp_path, host_only):
    text, want = _data_set(ref, tmp_path)
    data = pimc.BoxDataPM.from_json_string(text)
    data.preprocess()
    for k in ("beta", "tau", "beta_plus", "beta_minus", "tau_plus", "tau_minus"):
        assert np.isclose(getattr(data, k), float(want[k + "_pre"]), rtol=1e-15, atol=0), k
    params_scratch = os.path.join(str(tmp_path), f"data_set_{data.id_data}", f"rho_{data.id_rho}") + "/"
    FS = file_structure.FileStructure.from_boxdata(os.path.normpath(os.path.join(params_scratch, "../..")), data)
    result = pimc.BoxResultPM(data=data)
    result.path_root, result.id_job = FS.path_rho_results, "3"
    assert result.compute_path_to_file() == str(want["result_path"]).replace("@ROOT@", str(tmp_path))
    assert result.samples == int(want["samples"])
    assert np.all(np.isnan(result.scaled_gofr_plus))


def test_plain_box_ignores_the_plus_minus_step(ref, tmp_path, host_only):
    text, want = _data_set(ref, tmp_path)
    data = pimc.BoxData.from_json_string(text)
    assert data.delta_beta == float(want["delta_beta"])
    data.preprocess()
    assert not data._plus_minus()
    assert np.isclose(data.tau, float(want["tau_pre"]), rtol=1e-15, atol=0)


def test_too_few_beads_are_rejected(ref, tmp_path):
    text, _ = _data_set(ref, tmp_path)
    data = pimc.BoxDataPM.from_json_string(text)
    data.beads = 2
    with pytest.raises(AssertionError):
        data.preprocess()


def test_minimal_module_name_exports_the_engine():
    """examples/basic_ml_testing.py:17 of the reference imports the engine as pimc.minimal."""
    from pibronic_gb300 import minimal
    for name in ("BoxData", "BoxDataPM", "BoxResult", "BoxResultPM", "block_compute", "block_compute_pm",
                 "block_compute_gR_from_raw_samples", "block_compute_rhoR_from_input_samples",
                 "build_o_matrix", "build_numerator"):
        assert getattr(minimal, name) is getattr(pimc, name), name
