"""Seeded survey and records shared by the SeismicData format fixtures and their test.

``seismic_data_case(Source, Receiver, Survey, wavelet)`` builds the same survey with either the
reference's classes or this package's (both have the reference's API) and returns it with a
record dict of acoustic and elastic components.
"""
import numpy as np


def seismic_data_case(Source, Receiver, Survey, wavelet):
    nt, dt, f0 = 64, 2e-3, 12.0
    src = Source(nt=nt, dt=dt, f0=f0)
    _, wav = wavelet(nt, dt, f0)
    src.add_sources(src_x=np.array([3, 9, 15]), src_z=np.array([1, 1, 2]), src_wavelet=wav)
    src.add_source(7, 4, wav)
    rcv = Receiver(nt=nt, dt=dt)
    rcv.add_receivers(rcv_x=np.arange(0, 20, 2), rcv_z=np.full(10, 1), rcv_type="pr")
    rcv.add_receiver(5, 6, "vz")
    rng = np.random.default_rng(77)
    recs = {k: rng.standard_normal((4, nt, 11)).astype(np.float32) for k in ("p", "u", "w", "txx", "vx")}
    return Survey(src, rcv), recs
