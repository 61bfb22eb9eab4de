"""Result-file discovery and loading for the estimators (pibronic/data/postprocessing.py:48-58,
118-197, 294-340): which ``P*_T*_J*_data_points.npz`` files a data set holds, the bead counts and
temperatures they cover, hash pruning, and the merged load of all jobs of one (P, T).

File names follow ``file_structure.pimc`` / ``file_structure.jackknife``; parsing splits on the
same separators as the reference, so paths whose directories contain "P" or "_T" are read the
same way the reference reads them.
"""
from __future__ import annotations

import glob
import json

import numpy as np

from . import file_structure
from .analytic import load_analytic_data

__all__ = ["retrive_pimc_file_list", "retrive_jackknife_file_list", "extract_bead_paramater_list",
           "extract_temperature_paramater_list", "prune_results_using_hashes", "load_pimc_data",
           "load_analytic_data"]


def retrive_pimc_file_list(FS):
    """Every result file of the data set's sampling model (postprocessing.py:48-51)."""
    return list(glob.glob(FS.path_rho_results + file_structure.pimc(P="*", T="*", J="*")))


def retrive_jackknife_file_list(FS):
    """Every estimator output file (postprocessing.py:54-57)."""
    return list(glob.glob(FS.path_rho_results + file_structure.jackknife(P="*", T="*", X="*")))


def extract_bead_value_from_pimc_file_path(file_path):
    return int(file_path.split("P")[1].split("_T")[0])


def extract_bead_paramater_list(list_pimc):
    """Sorted unique bead counts (postprocessing.py:123-128)."""
    return sorted(set(map(extract_bead_value_from_pimc_file_path, list_pimc)))


def extract_temperature_value_from_pimc_file_path(file_path):
    return float(file_path.split("_T")[1].split("_J")[0])


def extract_temperature_paramater_list(list_pimc):
    """Sorted unique temperatures (postprocessing.py:136-144)."""
    return sorted(set(map(extract_temperature_value_from_pimc_file_path, list_pimc)))


def extract_job_value_from_pimc_file_path(file_path):
    return int(file_path.split("_J")[1].split("_data_")[0])


def extract_bead_value_from_thermo_file_path(file_path):
    return int(file_path.split("P")[1].split("_T")[0])


def extract_temperature_value_from_thermo_file_path(file_path):
    return float(file_path.split("_T")[1].split("_X")[0])


def extract_sample_value_from_thermo_file_path(file_path):
    return int(file_path.split("_X")[1].split("_thermo")[0])


def prune_results_using_hashes(FS, list_pimc):
    """The paths whose stored model hashes equal FS's (postprocessing.py:175-196): ``.npz`` result
    files and ``_thermo`` JSON files; any other suffix raises."""
    out = []
    for path in list_pimc:
        if path.endswith(".npz"):
            with np.load(path, mmap_mode="r") as f:
                if "hash_vib" not in f or "hash_rho" not in f:
                    continue
                if f["hash_vib"] == FS.hash_vib and f["hash_rho"] == FS.hash_rho:
                    out.append(path)
        elif path.endswith("thermo"):
            with open(path) as fh:
                data = json.loads(fh.read())
            if "hash_vib" not in data or "hash_rho" not in data:
                continue
            if data["hash_vib"] == FS.hash_vib and data["hash_rho"] == FS.hash_rho:
                out.append(path)
        else:
            raise Exception(f"file path {path:s} undefined")
    return out


def load_pimc_data(FS, P, T, pimc_results):
    """Merge every job's result file at (P, T) into `pimc_results` (postprocessing.py:294-310)."""
    pimc_results.load_multiple_results(list(glob.glob(FS.template_pimc.format(P=P, T=T, J="*"))))
