"""remove_coupling_from_model / create_harmonic_model / create_basic_diagonal_model
(vibronic_model_io.py:749-787) against the files the reference's own function wrote from the same
coupled models (tests/golden/make_golden.py): the same text, so the same model hash.  Host only."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from pibronic_gb300 import file_structure as fs, vibronic_io


@pytest.fixture(scope="module")
def derived():
    with np.load(os.path.join(GOLDEN, "reference_derived_models.npz")) as d:
        return {k: str(d[k]) for k in d.files}


def _names(derived):
    return sorted({k.rsplit("/", 1)[0] for k in derived})


def test_diagonal_model_text_matches_the_reference(derived, tmp_path):
    names = _names(derived)
    assert len(names) == 4
    for i, name in enumerate(names):
        src, dst = tmp_path / f"in_{i}.json", tmp_path / f"out_{i}.json"
        src.write_text(derived[name + "/coupled"])
        vibronic_io.remove_coupling_from_model(str(src), str(dst))
        assert dst.read_text() == derived[name + "/diagonal"], name
        assert vibronic_io.create_diagonal_model_hash(path=str(dst)) == vibronic_io._hash(derived[name + "/diagonal"])


def test_basic_diagonal_model_is_the_harmonic_model(derived, tmp_path):
    FS = fs.FileStructure(str(tmp_path), 1, 0)
    name = _names(derived)[0]
    with open(FS.path_vib_model, "w") as fh:
        fh.write(derived[name + "/coupled"])
    path = vibronic_io.create_basic_diagonal_model(FS)
    assert path == FS.path_rho_model
    with open(FS.path_har_model) as fh:
        har = fh.read()
    with open(FS.path_rho_model) as fh:
        assert fh.read() == har == derived[name + "/diagonal"]
