"""SEP regular-file I/O (the reference's genericIO dataset format)."""
import os

import numpy as np


def test_round_trip_xdr_and_native(born, tmp_path):
    rng = np.random.default_rng(0)
    a = rng.standard_normal((5, 6, 7)).astype(np.float32)
    for be in (True, False):
        p = str(tmp_path / f"v{int(be)}.H")
        born.write_sep(p, a, o=(1.0, 2.0, 3.0), d=(10.0, 11.0, 12.0),
                       big_endian=be)
        b, o, d = born.read_sep(p)
        assert np.array_equal(a, b)
        assert o == (1.0, 2.0, 3.0) and d == (10.0, 11.0, 12.0)
    # xdr data on disk is big-endian
    raw = np.fromfile(str(tmp_path / "v1.H@"), ">f4")
    assert np.array_equal(raw, a.ravel())


def test_hand_written_header(born, tmp_path):
    data = np.arange(24, dtype=">f4")
    data.tofile(str(tmp_path / "wav.bin"))
    hdr = tmp_path / "wav.H"
    hdr.write_text(
        "# written by a SEP program\n"
        "n1=10 o1=0 d1=.004 label1=\"time\"\n"
        "n1=12 n2=2 d2=25\n"              # later pairs override earlier ones
        'esize=4 data_format="xdr_float"\n'
        "in='wav.bin'\n")
    a, o, d = born.read_sep(str(hdr))
    assert a.shape == (2, 12)
    assert np.array_equal(a.ravel(), np.arange(24, dtype=np.float32))
    assert d == (np.float32(.004), 25.0)


def test_bad_headers_are_rejected(born, tmp_path):
    import pytest
    h = tmp_path / "x.H"
    h.write_text("n1=4 esize=8 in=x.bin\n")
    with pytest.raises(born.BornError):
        born.read_sep(str(h))
    h.write_text("n1=4 data_format=xdr_int in=x.bin\n")
    with pytest.raises(born.BornError):
        born.read_sep(str(h))
    h.write_text("n1=4 in=missing.bin\n")
    with pytest.raises(born.BornError):
        born.read_sep(str(h))
