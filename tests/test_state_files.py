"""FLEXI state files (io_hdf5/hdf5_output.f90 WriteState, restart.f90 ReadState) read and written
without libhdf5.

The reference's own state file (regressioncheck/checks/parabolic/cavity_3D, a fixture written by the
HDF5 library behind a 4 KB user block) is read, written back by dg_write_state and read again; the
object-header messages the writer produces for the same attributes and dataset are byte-identical to
the ones the HDF5 library wrote into the reference file.
"""
import os

import numpy as np
import pytest

import galaexi_gb300 as gx

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF = os.path.join(GOLDEN, "reggie_cavity_Re100_State_0000001.000000000.h5")


def written(tmp_path):
    U, t, N, nt, mf = gx.read_state(REF)
    out = tmp_path / "cavity_Re100_State_0000001.000000000.h5"
    gx.write_state(out, U, N, nt, t, mf, project="cavity_Re100")
    return out, U, t, N, nt, mf


def test_round_trip(tmp_path):
    out, U, t, N, nt, mf = written(tmp_path)
    U2, t2, N2, nt2, mf2 = gx.read_state(out)
    assert U2.shape == (64, 3, 3, 3, 5) and np.array_equal(U2, U)
    assert (t2, N2, nt2, mf2) == (t, N, nt, mf) == (1.0, 2, "GAUSS", "cavity4x4x4_mesh.h5")
    assert gx.read_h5(out, "File_Type", True) == "State"
    assert gx.read_h5(out, "Project_Name", True) == "cavity_Re100"
    assert float(gx.read_h5(out, "File_Version", True)[0]) == 0.1
    assert int(gx.read_h5(out, "Dimension", True)[0]) == 3
    assert gx.read_h5(out, "NextFile", True) == out.name


def message_bytes(path, name):
    """The bytes of the version-1 attribute message named `name` (8-byte message header included),
    found by its fixed layout: version 1, name length, then the NUL-terminated name."""
    data = open(path, "rb").read()
    key = bytes([1, 0, len(name) + 1, 0])  # version, reserved, name size (2 bytes)
    pos = 0
    while True:
        i = data.find(key, pos)
        assert i >= 0, name
        nm = data[i + 8:i + 8 + len(name) + 1]
        if nm == name.encode() + b"\0":
            size = int.from_bytes(data[i - 6:i - 4], "little")
            return data[i - 8:i + size]
        pos = i + 1


@pytest.mark.parametrize("attr", ["File_Type", "Project_Name", "File_Version", "VarNames", "N", "Dimension", "Time",
                                  "MeshFile"])
def test_attribute_messages_match_hdf5_library(tmp_path, attr):
    out, *_ = written(tmp_path)
    assert message_bytes(out, attr) == message_bytes(REF, attr)


def test_dataset_messages_match_hdf5_library(tmp_path):
    out, *_ = written(tmp_path)
    ref, mine = open(REF, "rb").read(), open(out, "rb").read()
    # dataspace (rank 5, maximum dimensions), IEEE double datatype and fill-value messages of
    # DG_Solution: type, size, flags, reserved, body
    dims = (64, 3, 3, 3, 5)
    space = bytes([1, 0, 88, 0, 0, 0, 0, 0, 1, 5, 1, 0, 0, 0, 0, 0]) + b"".join(
        d.to_bytes(8, "little") for d in dims * 2)
    dtype = bytes([3, 0, 24, 0, 1, 0, 0, 0]) + bytes.fromhex("11203f000800000000004000340b0034ff03000000000000")
    fill = bytes([5, 0, 8, 0, 1, 0, 0, 0]) + bytes.fromhex("0202020100000000")
    for blob in (space, dtype + fill):
        assert ref.find(blob) >= 0 and mine.find(blob) >= 0
