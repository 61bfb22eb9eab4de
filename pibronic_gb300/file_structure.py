"""Directory layout and file names of a data set (pibronic/data/file_structure.py:33-140,
pibronic/data/file_name.py:38-140): data_set_{D}/[rho_{R}/]{parameters,results,...}/ with model
files coupled_model.json / sampling_model.json and result files P{P}_T{T:.2f}_J{J}_data_points.npz."""
from __future__ import annotations

import os
from os.path import join

from . import vibronic_io as vIO

coupled_model = "coupled_model.json"
harmonic_model = "harmonic_model.json"
sampling_model = "sampling_model.json"
analytic_results = "analytic_results.json"


def pimc(P="{P:d}", T="{T:.2f}", J="{J:d}"):
    """Result file name of one job (file_name.py:38-46)."""
    return "P{:s}_T{:s}_J{:s}_data_points.npz".format(P, T, J)


def jackknife(P="{P:d}", T="{T:.2f}", X="{X:d}"):
    """Estimator output name (file_name.py:55-62)."""
    return "P{:s}_T{:s}_X{:s}_thermo".format(P, T, X)


def training_data_input(P="{P:d}", T="{T:.2f}", J="{J:d}"):
    return "P{:s}_T{:s}_J{:s}_training_data_input.npz".format(P, T, J)


def training_data_g_output(P="{P:d}", T="{T:.2f}", J="{J:d}"):
    return "P{:s}_T{:s}_J{:s}_training_data_g_output.npz".format(P, T, J)


def training_data_rho_output(P="{P:d}", T="{T:.2f}", J="{J:d}"):
    return "P{:s}_T{:s}_J{:s}_training_data_rho_output.npz".format(P, T, J)


class FileStructure:
    """Paths of one (data set, sampling model) pair; creates the directories unless told not to."""

    def __init__(self, path_root, id_data, id_rho=0, no_makedir=False):
        assert os.path.isdir(path_root), f"the path_root ({path_root}) is not a directory"
        self.id_data, self.id_rho = id_data, id_rho
        self.path_root = os.path.abspath(path_root)
        vib = join(self.path_root, f"data_set_{id_data:d}")
        rho = join(vib, f"rho_{id_rho:d}")
        self.path_data, self.path_rho = vib + "/", rho + "/"
        self.path_vib_params = join(vib, "parameters") + "/"
        self.path_vib_results = join(vib, "results") + "/"
        self.path_vib_output = join(vib, "execution_output") + "/"
        self.path_vib_plots = join(vib, "plots") + "/"
        self.path_rho_params = join(rho, "parameters") + "/"
        self.path_rho_results = join(rho, "results") + "/"
        self.path_rho_output = join(rho, "execution_output") + "/"
        self.path_rho_plots = join(rho, "plots") + "/"
        self.dir_list = [k for k in vars(self) if k.startswith("path_") and k != "path_root"]
        self.template_pimc = self.path_rho_results + pimc(J="{J:s}")
        self.template_jackknife = self.path_rho_results + jackknife()
        self.path_vib_model = join(self.path_vib_params, coupled_model)
        self.path_har_model = join(self.path_vib_params, harmonic_model)
        self.path_rho_model = join(self.path_rho_params, sampling_model)
        self.path_analytic_rho = join(self.path_rho_params, analytic_results)
        if not no_makedir:
            self.make_directories()

    @classmethod
    def from_boxdata(cls, path_root, data):
        return cls(path_root, data.id_data, data.id_rho)

    def make_directories(self):
        for attr in self.dir_list:
            os.makedirs(getattr(self, attr), exist_ok=True)

    def directories_exist(self):
        return all(os.path.isdir(getattr(self, a)) for a in self.dir_list)

    def generate_model_hashes(self, force_flag=False):
        if hasattr(self, "hash_vib") and hasattr(self, "hash_rho") and not force_flag:
            return
        self.hash_vib = vIO.create_model_hash(FS=self)
        self.hash_rho = vIO.create_diagonal_model_hash(FS=self)
