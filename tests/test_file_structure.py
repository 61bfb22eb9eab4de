"""The data-set directory layout as the reference's own test states it
(tests/data/test_file_structure.py of the reference, file_structure.py:31-207), on this package's
FileStructure.  Host only."""
import os
from os.path import join, samefile

import pytest

from pibronic_gb300 import file_structure as fs


def test_FileStructure_directory_creation(tmp_path):
    root = tmp_path / "root"
    root.mkdir()
    id_data, id_rho = 0, 0
    FS = fs.FileStructure(str(root), id_data, id_rho)
    dict_path = {
        "path_root": "",
        "path_data": f"data_set_{id_data}",
        "path_es": f"data_set_{id_data}/electronic_structure",
        "path_vib_params": f"data_set_{id_data}/parameters",
        "path_vib_results": f"data_set_{id_data}/results",
        "path_vib_output": f"data_set_{id_data}/execution_output",
        "path_vib_plots": f"data_set_{id_data}/plots",
        "path_rho": f"data_set_{id_data}/rho_{id_rho}",
        "path_rho_params": f"data_set_{id_data}/rho_{id_rho}/parameters",
        "path_rho_results": f"data_set_{id_data}/rho_{id_rho}/results",
        "path_rho_output": f"data_set_{id_data}/rho_{id_rho}/execution_output",
        "path_rho_plots": f"data_set_{id_data}/rho_{id_rho}/plots",
    }
    for key, value in dict_path.items():
        assert samefile(getattr(FS, key), join(str(root), value)), key
    assert FS.directories_exist()
    # file paths are not created as directories
    assert not os.path.exists(FS.path_rho_model) and not os.path.exists(FS.path_analytic_rho)


def test_file_templates(tmp_path):
    FS = fs.FileStructure(str(tmp_path), 2, 1)
    assert FS.template_pimc.format(P=12, T=300.0, J="*").endswith("data_set_2/rho_1/results/P12_T300.00_J*_data_points.npz")
    assert FS.template_jackknife.format(P=8, T=250.0, X=30).endswith("rho_1/results/P8_T250.00_X30_thermo")
    assert FS.template_sos_rho.format(B=80).endswith("rho_1/parameters/sos_B80.json")
    assert FS.template_sos_vib.format(B=60).endswith("data_set_2/parameters/sos_B60.json")
    assert FS.template_trotter_vib.format(P=16, B=80).endswith("parameters/trotter_P16_B80.json")
    assert FS.path_vib_model.endswith("data_set_2/parameters/coupled_model.json")
    assert FS.path_rho_model.endswith("data_set_2/rho_1/parameters/sampling_model.json")


def test_change_rho_moves_the_sampling_paths(tmp_path):
    FS = fs.FileStructure(str(tmp_path), 0, 0)
    FS.change_rho(3)
    assert os.path.isdir(join(str(tmp_path), "data_set_0", "rho_3", "results"))
    assert FS.path_rho_results.endswith("data_set_0/rho_3/results/")
    assert FS.path_rho_model.endswith("rho_3/parameters/sampling_model.json")
    assert FS.template_pimc.startswith(FS.path_rho_results)


def test_no_makedir_and_missing_root(tmp_path):
    FS = fs.FileStructure(str(tmp_path), 4, 5, no_makedir=True)
    assert not FS.directories_exist()
    with pytest.raises(AssertionError):
        fs.FileStructure(str(tmp_path / "absent"), 0, 0)
