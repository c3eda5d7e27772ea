"""Keras weight-file import without h5py (nerf/core/model.py:278-287 loads
the files nerf/core/ops.py:142-143 writes).

The reader is pinned on a real HDF5 file written by the HDF5 library: SciPy's
MATLAB v7.3 test file, whose variable SciPy's own tests state as
testdouble = pi/4 * arange(9). The Keras layout (layer_names, weight_names,
nested weight datasets) is checked on files from tests/h5_writer.py, which
follows the format specification with the HDF5 library's default structures;
no real Keras checkpoint or h5py is available to check it against."""
import importlib
import os
import struct

import numpy as np
import pytest

import h5_writer

MAT = os.path.join(os.path.dirname(np.__file__), "..", "scipy", "io", "matlab", "tests", "data",
                   "testhdf5_7.4_GLNX86.mat")


def h5(ng):
    return importlib.import_module("nerf-tf2_gb300.h5")


def test_reads_a_real_hdf5_file(ng):
    """SciPy's test file (MATLAB, HDF5 library 1.8, a 512-byte user block):
    superblock version 0, a symbol-table root group, one contiguous float64
    dataset with a fixed-length string attribute."""
    if not os.path.exists(MAT):
        pytest.skip("SciPy's MATLAB test data are not installed")
    root = h5(ng).open_file(MAT)
    assert list(root.members()) == ["testdouble"]
    ds = root["testdouble"]
    assert ds.shape == (9, 1) and ds.dtype == np.float64
    # SciPy's expectation for this variable (scipy/io/matlab/tests/test_mio.py)
    assert np.array_equal(ds.read(), (np.pi / 4 * np.arange(9, dtype=float)).reshape(9, 1))
    assert ds.attrs["MATLAB_class"] == b"double"


def keras_layers(ng, model_name, blob):
    """The reference network's layers in Keras order, with weights for the
    Dense layers (weight names as Keras gives them)."""
    d = ng.weights.to_dict(blob, model_name)
    m = model_name
    order = [f"{m}/xyz", f"{m}/rays_d", f"{m}/enc_xyz", f"{m}/enc_rays_d"] + \
            [f"{m}/dense_{i}" for i in range(5)] + [f"{m}/concat_1"] + \
            [f"{m}/dense_{i}" for i in (5, 6, 7)] + [f"{m}/sigma", f"{m}/dense_8", f"{m}/concat_2",
                                                       f"{m}/dense_9", f"{m}/rgb"]
    out = []
    for lname in order:
        short = lname.split("/", 1)[1]
        if f"{m}/{short}/kernel:0" in d:
            out.append((lname, [(f"{lname}/kernel:0", d[f"{m}/{short}/kernel:0"]),
                                (f"{lname}/bias:0", d[f"{m}/{short}/bias:0"])]))
        else:
            out.append((lname, []))
    return out


@pytest.mark.parametrize("model_name,split,userblock", [("coarse", False, 0), ("fine", True, 512)])
def test_keras_weight_file_roundtrip(ng, tmp_path, model_name, split, userblock):
    blob = ng.weights.glorot_blob(17)
    blob[ng.weights.offsets()["rgb"][1]:][:3] = [0.25, -0.5, 1.0]  # non-zero biases too
    layers = keras_layers(ng, model_name, blob)
    p = str(tmp_path / f"x_{model_name}.h5")
    h5_writer.write_keras_weights(p, layers, split_layer_names=split, userblock=userblock)
    got = h5(ng).keras_layer_weights(p)
    assert [ln for ln, _ in got] == [ln for ln, ws in layers if ws]
    d = ng.weights.from_keras_layers(got, model_name)
    assert np.array_equal(ng.weights.from_dict(d, model_name), blob)
    # the root: more than 2K = 8 members, so several symbol table nodes
    root = h5(ng).open_file(p)
    assert len(root[model_name].members()) == len(layers) > 8
    assert h5(ng).keras_attribute(root, "layer_names") == [ln for ln, _ in layers]
    assert root.attrs["backend"] == b"tensorflow"


def test_keras_weights_checked(ng, tmp_path):
    blob = ng.weights.glorot_blob(3)
    layers = keras_layers(ng, "coarse", blob)
    lname, ws = layers[5]  # coarse/dense_1
    layers[5] = (lname, [(ws[0][0], ws[0][1][:, :128]), ws[1]])
    p = str(tmp_path / "bad.h5")
    h5_writer.write_keras_weights(p, layers)
    with pytest.raises(ValueError, match="shapes"):
        ng.weights.from_keras_layers(h5(ng).keras_layer_weights(p), "coarse")
    with pytest.raises(ValueError, match="layers with weights"):
        ng.weights.from_keras_layers(h5(ng).keras_layer_weights(p)[:-1], "coarse")


def test_refuses_what_it_does_not_read(ng, tmp_path):
    p = tmp_path / "v2.h5"
    p.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes([2, 8, 8, 0]) + b"\0" * 64)
    with pytest.raises(NotImplementedError, match="superblock version 2"):
        h5(ng).open_file(str(p))
    q = tmp_path / "not.h5"
    q.write_bytes(b"not an hdf5 file" * 64)
    with pytest.raises(h5(ng).H5Error):
        h5(ng).open_file(str(q))
    # a version-2 object header ("OHDR") where the root's should be
    w = h5_writer.Writer()
    root = w.group({})
    w.close(str(tmp_path / "o.h5"), root)
    data = bytearray((tmp_path / "o.h5").read_bytes())
    data[root[1]:root[1] + 4] = b"OHDR"
    (tmp_path / "o.h5").write_bytes(bytes(data))
    with pytest.raises(NotImplementedError, match="version-2 object headers"):
        h5(ng).open_file(str(tmp_path / "o.h5"))


def test_attribute_and_dataset_types(ng, tmp_path):
    w = h5_writer.Writer()
    ds = {"f4": np.arange(6, dtype=np.float32).reshape(2, 3), "f8": np.linspace(0, 1, 5),
          "i4": np.array([-3, 7], np.int32), "u2": np.array([1, 65535], np.uint16)}
    members = {k: w.dataset(v, attrs={"unit": np.bytes_(b"m"), "n": np.array([1, 2], np.int64)})
               for k, v in ds.items()}
    root = w.group(members, attrs={"scalar": np.float64(2.5), "empty": np.asarray([])})
    w.close(str(tmp_path / "t.h5"), root)
    r = h5(ng).open_file(str(tmp_path / "t.h5"))
    for k, v in ds.items():
        got = r[k].read()
        assert got.dtype == v.dtype and np.array_equal(got, v), k
        assert r[k].attrs["unit"] == b"m" and np.array_equal(r[k].attrs["n"], [1, 2])
    assert r.attrs["scalar"] == 2.5 and r.attrs["empty"].shape == (0,)
    with pytest.raises(KeyError):
        r["missing"]
    assert "f4" in r and "nope" not in r
    assert struct.unpack_from("<I", (tmp_path / "t.h5").read_bytes(), 8)[0] & 0xFF == 0  # superblock v0


def test_model_entry_points(ng, tmp_path):
    """NerfMLP.load_weights reads the file into set_weights (Keras names of
    the network it is called on); NeRF.load_model loads <tag>_coarse.h5 and
    <tag>_fine.h5 from the directory (model.py:278-287). Called on host
    stand-ins: constructing the real objects needs a device."""
    blob = ng.weights.glorot_blob(5)
    h5_writer.write_keras_weights(str(tmp_path / "000100_31.20_coarse.h5"), keras_layers(ng, "coarse", blob))
    h5_writer.write_keras_weights(str(tmp_path / "000100_31.20_fine.h5"), keras_layers(ng, "fine", blob[::-1].copy()))

    class FakeMLP:
        def __init__(self, name):
            self.name, self.got = name, None

        def set_weights(self, d):
            self.got = ng.weights.from_dict(d, self.name)

        def load_weights(self, path):
            ng.model.NerfMLP.load_weights(self, path)

    class FakeNeRF:
        coarse_model, fine_model = FakeMLP("coarse"), FakeMLP("fine")

    fake = FakeNeRF()
    ng.model.NeRF.load_model(fake, str(tmp_path), "000100_31.20")
    assert np.array_equal(fake.coarse_model.got, blob)
    assert np.array_equal(fake.fine_model.got, blob[::-1])
