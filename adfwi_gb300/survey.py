"""Acquisition geometry with the reference's API.

Mirrors ``ADFWI/survey``: ``Source`` (source.py:20-158: integer grid coordinates, one wavelet
row and one 3x3 moment tensor per source), ``Receiver`` (receiver.py:18-112: receivers shared
by every shot), ``Survey`` (survey.py:21-56) and ``SeismicData`` (data.py:22-170: npz I/O of
the record dict, byte-compatible with the reference's ``save`` / ``load``). Plotting methods
are not part of this package.
"""
from typing import List, Optional

import numpy as np

from .utils import gpu2cpu, list2numpy, numpy2list, tensor2numpy

_DEFAULT_MT = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1]])


class Source(object):
    """Seismic sources: grid positions (cells), wavelets (nsrc, nt) and moment tensors (nsrc, 3, 3)."""

    def __init__(self, nt: int, dt: float, f0: float) -> None:
        self.nt = nt
        self.dt = dt
        self.f0 = f0
        self.t = np.arange(nt) * dt
        self.loc_x, self.loc_z, self.loc = [], [], []
        self.type, self.wavelet, self.moment_tensor = [], [], []
        self.num = 0

    def __repr__(self):
        if self.num == 0:
            return "Seismic Source:\n  empty\n"
        x, z = list2numpy(self.loc_x), list2numpy(self.loc_z)
        return ("Seismic Source:\n"
                f"  Source wavelet: {self.nt} samples at {self.dt * 1000:.2f} ms\n"
                f"  Source number : {self.num}\n"
                f"  Source types  : {self.get_type(unique=True)}\n"
                f"  Source x range: {x.min()} - {x.max()} (grids)\n"
                f"  Source z range: {z.min()} - {z.max()} (grids)\n")

    def _validate(self, src_type, src_wavelet, src_mt):
        if src_type.lower() not in ["mt"]:
            raise ValueError("Source type must be either mt")
        if src_wavelet.shape[0] != self.nt:
            raise ValueError("Source wavelet must have the same length as the number of time samples")
        if src_mt is None:
            raise ValueError("Moment tensor must be provided for mt source")
        if src_mt.shape != (3, 3):
            raise ValueError("Moment tensor must be a 3x3 matrix")

    def add_sources(self, src_x: np.ndarray, src_z: np.ndarray, src_wavelet: np.ndarray,
                    src_type: Optional[str] = "mt", src_mt: Optional[np.ndarray] = _DEFAULT_MT) -> None:
        """Add several sources that share one wavelet and one moment tensor."""
        if src_x.shape != src_z.shape:
            raise ValueError("Source location along x and z direction must have the same shape")
        self._validate(src_type, src_wavelet, src_mt)
        n = len(src_x)
        self.loc_x.extend(numpy2list(src_x.reshape(-1)))
        self.loc_z.extend(numpy2list(src_z.reshape(-1)))
        self.type.extend([src_type] * n)
        self.wavelet.extend(np.ones((n, self.nt)) * src_wavelet)
        self.moment_tensor.extend(np.ones((n, 3, 3)) * src_mt)
        self.num += n

    def add_source(self, src_x: int, src_z: int, src_wavelet: np.ndarray, src_type: Optional[str] = "mt",
                   src_mt: Optional[np.ndarray] = _DEFAULT_MT) -> None:
        self._validate(src_type, src_wavelet, src_mt)
        self.loc_x.append(src_x)
        self.loc_z.append(src_z)
        self.type.append(src_type)
        self.wavelet.append(src_wavelet)
        self.moment_tensor.append(src_mt)
        self.num += 1

    def get_loc(self):
        loc = np.hstack((list2numpy(self.loc_x).reshape(-1, 1), list2numpy(self.loc_z).reshape(-1, 1)))
        self.loc = loc.copy()
        return loc

    def get_wavelet(self):
        return list2numpy(self.wavelet)

    def get_moment_tensor(self):
        return list2numpy(self.moment_tensor)

    def get_type(self, unique=False) -> List[str]:
        return list2numpy(list(set(self.type))) if unique else list2numpy(self.type)


class Receiver(object):
    """Receivers (grid cells), shared by all shots."""

    def __init__(self, nt: int, dt: float) -> None:
        self.nt = nt
        self.dt = dt
        self.loc_x, self.loc_z, self.locs, self.type = [], [], [], []
        self.num = 0

    def __repr__(self):
        if self.num == 0:
            return "Seismic Receiver:\n  empty\n"
        x, z = np.array(self.loc_x), np.array(self.loc_z)
        return ("Seismic Receiver:\n"
                f"  Receiver data   : {self.nt} samples at {self.dt * 1000:.2f} ms\n"
                f"  Receiver number : {self.num}\n"
                f"  Receiver types  : {self.get_type(unique=True)}\n"
                f"  Receiver x range: {x.min()} - {x.max()} (grids)\n"
                f"  Receiver z range: {z.min()} - {z.max()} (grids)\n")

    def add_receivers(self, rcv_x: np.ndarray, rcv_z: np.ndarray, rcv_type: str) -> None:
        if rcv_x.shape != rcv_z.shape:
            raise ValueError("Receiver Error: Inconsistant number of receiver in X and Z directions")
        if rcv_type.lower() not in ["pr", "vx", "vz"]:
            raise ValueError("Receiver type must be either pr, vx, vz")
        n = len(rcv_x)
        self.loc_x.extend(numpy2list(rcv_x.reshape(-1)))
        self.loc_z.extend(numpy2list(rcv_z.reshape(-1)))
        self.type.extend([rcv_type] * n)
        self.num += n

    def add_receiver(self, rcv_x: int, rcv_z: int, rcv_type: str) -> None:
        if rcv_type.lower() not in ["pr", "vx", "vz"]:
            raise ValueError("Receiver type must be either pr, vx, vz")
        self.loc_x.append(rcv_x)
        self.loc_z.append(rcv_z)
        self.type.append(rcv_type)
        self.num += 1

    def get_loc(self):
        loc = np.hstack((list2numpy(self.loc_x).reshape(-1, 1), list2numpy(self.loc_z).reshape(-1, 1)))
        self.loc = loc.copy()
        return loc

    def get_type(self, unique=False) -> List[str]:
        return list2numpy(list(set(self.type))) if unique else list2numpy(self.type)


class Survey(object):
    """Sources plus receivers; every source sees the same receivers, nt and dt."""

    def __init__(self, source: Source, receiver: Receiver) -> None:
        self.source = source
        self.receiver = receiver

    def __repr__(self):
        return "Survey Information:\n" + repr(self.source) + "\n" + repr(self.receiver)


class SeismicData(object):
    """Shot-gather container with npz save / load in the reference's layout."""

    def __init__(self, survey: Survey):
        self.survey = survey
        self.src_num = survey.source.num
        self.rcv_num = survey.receiver.num
        self.src_loc = survey.source.get_loc()
        self.rcv_loc = survey.receiver.get_loc()
        self.src_type = survey.source.get_type()
        self.rcv_type = survey.receiver.get_type()
        self.nt = survey.receiver.nt
        self.dt = survey.receiver.dt
        self.t = np.arange(self.nt) * self.dt
        self.data = None

    def __repr__(self):
        return ("Seismic Data:\n"
                f"  Source number : {self.src_num}\n"
                f"  Receiver number : {self.rcv_num}\n"
                f"  Time samples : {self.nt} samples at {self.dt * 1000:.2f} ms\n")

    def record_data(self, data: dict):
        for key, value in data.items():
            data[key] = tensor2numpy(gpu2cpu(value)).copy()
        self.data = data

    def save(self, path: str):
        np.savez(path, data=self.data, src_loc=self.src_loc, rcv_loc=self.rcv_loc, src_num=self.src_num,
                 rcv_num=self.rcv_num, rcv_type=self.rcv_type, src_type=self.src_type, t=self.t,
                 nt=self.nt, dt=self.dt)

    def load(self, path: str):
        d = np.load(path, allow_pickle=True)
        self.data = d["data"].item()
        self.src_loc = d["src_loc"]
        self.rcv_loc = d["rcv_loc"]
        self.src_num = d["src_num"]
        self.rcv_num = d["rcv_num"]
        self.rcv_type = d["rcv_type"]
        self.src_type = d["src_type"]
        self.t = d["t"]
        self.nt = d["nt"]
        self.dt = d["dt"]

    @staticmethod
    def _peak_normalised(a):
        return a / np.max(np.abs(a), axis=1, keepdims=True)

    def parse_elastic_data(self, normalize=False):
        """(pressure = -(txx + tzz), txz, vx, vz) of elastic records, each optionally divided by
        its traces' max |value| along time (data.py:100-113)."""
        d = self.data
        out = [-(d["txx"] + d["tzz"]), d["txz"], d["vx"], d["vz"]]
        return tuple(self._peak_normalised(a) for a in out) if normalize else tuple(out)

    def parse_acoustic_data(self, normalize=False):
        """(p, u, w) of acoustic records, optionally trace-normalised (data.py:115-123)."""
        out = [self.data["p"], self.data["u"], self.data["w"]]
        return tuple(self._peak_normalised(a) for a in out) if normalize else tuple(out)
