"""petgem_gb300.hdf5: the result-file writer used when h5py is absent.

* The reader parses petgem's own h5py-written tests/data/receiver_pos.h5
  (copied unchanged to tests/golden/petgem_receiver_pos.h5).
* For a float64 (58, 3) dataset the writer produces the dataspace, datatype
  and fill-value messages byte for byte as h5py wrote them in that file.
* Every kind of value petgem writes (strings, ints, bools, floats, float and
  complex arrays) round-trips, including groups of more than 8 entries
  (several symbol-table nodes) and nested groups.
* The structures follow the classic format: signatures, the version-0
  superblock with the end-of-file address, sorted symbol-table nodes whose
  B-tree keys are the last names, and a local heap with its free block.
"""
import os
import struct

import numpy as np

from petgem_gb300 import hdf5
from tests.helpers import GOLDEN

REF = os.path.join(GOLDEN, "petgem_receiver_pos.h5")


def _dataset_messages(b, hdr):
    msgs = hdf5._read_object(b, hdr)
    out = {}
    for t, at in msgs.items():
        n = struct.unpack_from("<H", b, at - 6)[0]
        out[t] = b[at:at + n]
    return out


def _root_entries(b):
    root = struct.unpack_from("<Q", b, 0x40)[0]
    bt, hp = struct.unpack_from("<QQ", b, hdf5._read_object(b, root)[0x11])
    return hdf5._group_entries(b, bt, hp), bt, hp


def test_reads_petgems_h5py_file():
    d = hdf5.read(REF)
    assert list(d) == ["data"]
    a = d["data"]
    assert a.shape == (58, 3) and a.dtype == np.float64
    assert np.allclose(a[0], [58.3333, 1750.0, -990.0]) and np.allclose(a[-1], [3383.3333, 1750.0, -990.0])
    assert np.all(np.diff(a[:, 0]) > 0)


def test_float_dataset_messages_match_h5py(tmp_path):
    ref = open(REF, "rb").read()
    (_, ref_hdr), = _root_entries(ref)[0]
    p = hdf5.write(str(tmp_path / "t.h5"), {"data": np.zeros((58, 3))})
    mine = open(p, "rb").read()
    (_, my_hdr), = _root_entries(mine)[0]
    a, b = _dataset_messages(ref, ref_hdr), _dataset_messages(mine, my_hdr)
    for t in (0x0001, 0x0003, 0x0005):          # dataspace, datatype, fill value
        assert a[t] == b[t], hex(t)
    assert b[0x0008][:2] == bytes([3, 1])        # contiguous layout, version 3
    assert struct.unpack_from("<Q", b[0x0008], 10)[0] == 58 * 3 * 8


def test_round_trip_of_petgem_result_values(tmp_path):
    ds = {
        "machine/machine": "node. 6.1.0. aarch64",
        "machine/num_processors": 1,
        "machine/petgem_version": "1.0",
        "model/date": "2026-12-04T12:00:00",
        "model/nord": 2,
        "model/dof": np.int64(1276096),
        "model/cuda": True,
        "model/vtk": False,
        "model/run-time (s)": 1.25,
        "model/sigma_horizontal (S/m)": np.array([3.3, 1.0, 0.01]),
        "model/frequency (Hz)": 1.0,
        "model/source_position (m)": np.array([0.0, 0.0, 50.0]),
        "model/polarization": np.array(["x", "y"]),
        "model/E-fields/x": np.array([1 + 2j, 3 - 4j, -5e-12 + 1e-13j]),
        "model/E-fields/y": np.zeros(3, complex),
    }
    for i in range(20):                          # more than one symbol-table node in "model"
        ds[f"model/extra {i:02d}"] = float(i) / 7.0
    p = hdf5.write(str(tmp_path / "csem_petgemV1.0_2026-12-04.h5"), ds)
    r = hdf5.read(p)
    assert set(r) == set(ds)
    for k, v in ds.items():
        if isinstance(v, str):
            assert r[k] == v, k
        else:
            got = np.asarray(r[k])
            assert got.dtype.kind == np.asarray(v).dtype.kind or np.asarray(v).dtype.kind == "U", k
            assert np.array_equal(got, np.asarray(v)), k


def test_structures_follow_the_classic_format(tmp_path):
    names = [f"n{i:02d}" for i in range(19)]
    p = hdf5.write(str(tmp_path / "s.h5"), {f"g/{n}": float(i) for i, n in enumerate(names)})
    b = open(p, "rb").read()
    assert b[:8] == hdf5.SIGNATURE and b[8] == 0
    assert struct.unpack_from("<Q", b, 0x28)[0] == len(b)          # end-of-file address
    (gname, ghdr), = _root_entries(b)[0]
    assert gname == "g"
    bt, hp = struct.unpack_from("<QQ", b, hdf5._read_object(b, ghdr)[0x11])
    assert b[bt:bt + 4] == b"TREE" and b[hp:hp + 4] == b"HEAP"
    used = struct.unpack_from("<H", b, bt + 6)[0]
    assert used == 3                                                # 19 names / 8 per node
    heap_size, free, data = struct.unpack_from("<QQQ", b, hp + 8)
    assert free < heap_size and struct.unpack_from("<QQ", b, data + free) == (1, 16)
    keys = [struct.unpack_from("<Q", b, bt + 24 + 16 * i)[0] for i in range(used + 1)]
    name_at = lambda off: b[data + off:b.index(b"\0", data + off)].decode()
    assert keys[0] == 0 and name_at(0) == ""
    entries = hdf5._group_entries(b, bt, hp)
    assert [e[0] for e in entries] == sorted(names)
    for i in range(used):                        # key i+1 = last name of child i
        child = struct.unpack_from("<Q", b, bt + 24 + 8 + 16 * i)[0]
        assert b[child:child + 4] == b"SNOD"
        n = struct.unpack_from("<H", b, child + 6)[0]
        last = struct.unpack_from("<Q", b, child + 8 + 40 * (n - 1))[0]
        assert keys[i + 1] == last


def test_write_results_uses_petgems_file_name(tmp_path):
    from petgem_gb300.pipeline import write_results
    stem = str(tmp_path / "csem_petgemV1.0_2026-12-04")
    path = write_results(stem, {"model/E-fields/x": np.array([1j, 2.0])})
    assert path == stem + ".h5" and os.path.exists(path)
    try:
        import h5py                                  # noqa: F401
    except ImportError:
        assert np.array_equal(hdf5.read(path)["model/E-fields/x"], np.array([1j, 2.0]))
