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


# model.layers of get_coarse_or_fine_model (model.py:334-394) as a Keras
# functional model lists them: by graph depth from the inputs, so the sigma
# head (an output) comes last and rays_d joins just before dense_8.
KERAS_ORDER = ["xyz", "enc_xyz"] + [f"dense_{i}" for i in range(5)] + ["concat_1"] + \
    [f"dense_{i}" for i in (5, 6, 7)] + ["rays_d", "dense_8", "enc_rays_d", "concat_2", "dense_9", "rgb", "sigma"]


def keras_layers(ng, model_name, blob, order=None):
    """The reference network's layers in the order Keras saves them (or
    `order`, short names), with weights for the Dense layers (weight names
    as Keras gives them)."""
    d = ng.weights.to_dict(blob, model_name)
    m = model_name
    order = [f"{m}/{s}" for s in (order or KERAS_ORDER)]
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


def test_load_order_does_not_depend_on_file_order(ng, tmp_path):
    """The file's layers are matched to the network's by name: the order of
    layer_names (Keras's depth order, the source order, or any other) gives
    the same blob."""
    blob = ng.weights.glorot_blob(23)
    source_order = ["xyz", "rays_d", "enc_xyz", "enc_rays_d"] + [f"dense_{i}" for i in range(5)] + \
        ["concat_1", "dense_5", "dense_6", "dense_7", "sigma", "dense_8", "concat_2", "dense_9", "rgb"]
    shuffled = list(KERAS_ORDER)
    np.random.default_rng(4).shuffle(shuffled)
    for k, order in enumerate((KERAS_ORDER, source_order, shuffled)):
        p = str(tmp_path / f"o{k}.h5")
        h5_writer.write_keras_weights(p, keras_layers(ng, "fine", blob, order))
        got = h5(ng).keras_layer_weights(p)
        assert [ln.split("/", 1)[1] for ln, _ in got] == [s for s in order if s.startswith(("dense", "sigma", "rgb"))]
        assert np.array_equal(ng.weights.from_dict(ng.weights.from_keras_layers(got, "fine"), "fine"), blob)


def test_keras_weights_checked(ng, tmp_path):
    blob = ng.weights.glorot_blob(3)
    layers = keras_layers(ng, "coarse", blob)
    k = [ln for ln, _ in layers].index("coarse/dense_1")
    lname, ws = layers[k]
    layers[k] = (lname, [(ws[0][0], ws[0][1][:, :128]), ws[1]])
    p = str(tmp_path / "bad.h5")
    h5_writer.write_keras_weights(p, layers)
    with pytest.raises(ValueError, match="shapes"):
        ng.weights.from_keras_layers(h5(ng).keras_layer_weights(p), "coarse")
    with pytest.raises(ValueError, match="layers with weights"):
        ng.weights.from_keras_layers(h5(ng).keras_layer_weights(p)[:-1], "coarse")
    q = str(tmp_path / "good.h5")
    h5_writer.write_keras_weights(q, keras_layers(ng, "coarse", blob))
    good = h5(ng).keras_layer_weights(q)
    renamed = [(ln.replace("dense_3", "dense_33"), ws) for ln, ws in good]
    with pytest.raises(ValueError, match="no layer coarse/dense_3"):
        ng.weights.from_keras_layers(renamed, "coarse")
    twice = [(ln.replace("dense_3", "dense_2"), ws) for ln, ws in good]
    with pytest.raises(ValueError, match="twice"):
        ng.weights.from_keras_layers(twice, "coarse")


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
        opt = None

        def load_optimizer_state(self, st):
            self.opt = st

    fake = FakeNeRF()
    ng.model.NeRF.load_model(fake, str(tmp_path), "000100_31.20", skip_optimizer=True)
    assert np.array_equal(fake.coarse_model.got, blob)
    assert np.array_equal(fake.fine_model.got, blob[::-1])
    assert fake.opt is None
    with pytest.raises(FileNotFoundError):  # as np.load in the reference's set_everything
        ng.model.NeRF.load_model(fake, str(tmp_path), "000100_31.20")
    m = {"coarse": blob * 0.5, "fine": blob * 0.25}
    v = {"coarse": blob * blob, "fine": blob * blob * 2}
    save_optimizer_npz(ng, str(tmp_path / "000100_31.20_optimizer.npz"), 1234, m, v)
    ng.model.NeRF.load_model(fake, str(tmp_path), "000100_31.20")
    assert fake.opt["step"] == 1234
    for name in ("coarse", "fine"):
        assert np.array_equal(fake.opt["m"][name], m[name].astype(np.float32))
        assert np.array_equal(fake.opt["v"][name], v[name].astype(np.float32))


def keras_adam_names(ng):
    """optimizer.variables() names of the reference's Keras Adam over the
    NeRF's trainable variables (coarse model's, then fine model's): the step
    count, the float hyperparameters, then every m slot and every v slot."""
    var = [f"{m}/{name}/{kind}" for m in ("coarse", "fine") for name, _, _ in ng.weights.LAYERS
           for kind in ("kernel", "bias")]
    return (["Adam/iter:0", "Adam/beta_1:0", "Adam/beta_2:0", "Adam/decay:0"] +
            [f"Adam/{x}/m:0" for x in var] + [f"Adam/{x}/v:0" for x in var])


def save_optimizer_npz(ng, path, step, m, v):
    """Writes the file as the reference's checkpoint callback does
    (nerf/core/ops.py:110-120): np.savez of {name: value} plus "names"."""
    off = ng.weights.offsets()
    items = {}
    for n in keras_adam_names(ng):
        if n == "Adam/iter:0":
            items[n] = np.int64(step)
        elif n.endswith(("beta_1:0", "beta_2:0", "decay:0")):
            items[n] = np.float32({"beta_1": 0.9, "beta_2": 0.999, "decay": 0.0}[n[5:-2]])
        else:
            _, model, layer, kind, slot = n[:-2].split("/")
            ko, bo, i, o = off[layer]
            src = (m if slot == "m" else v)[model]
            items[n] = src[ko:ko + i * o].reshape(i, o) if kind == "kernel" else src[bo:bo + o]
    items["names"] = np.array(keras_adam_names(ng))
    np.savez(path, **items)


def test_optimizer_npz_checked(ng, tmp_path):
    blob = ng.weights.glorot_blob(8)
    p = str(tmp_path / "x_optimizer.npz")
    save_optimizer_npz(ng, p, 7, {"coarse": blob, "fine": blob}, {"coarse": blob ** 2, "fine": blob ** 2})
    st = ng.weights.optimizer_state_from_npz(p)
    assert st["step"] == 7 and st["m"]["fine"].shape == (ng.weights.PARAM_COUNT,)
    d = dict(np.load(p))
    d["Adam/beta_1:0"] = np.float32(0.8)
    np.savez(p, **d)
    with pytest.raises(ValueError, match="beta_1"):
        ng.weights.optimizer_state_from_npz(p)
    d["Adam/beta_1:0"] = np.float32(0.9)
    d["names"] = np.array([n for n in d["names"] if n != "Adam/fine/rgb/bias/v:0"])
    np.savez(p, **d)
    with pytest.raises(ValueError, match="no Adam slot v for fine/rgb/bias"):
        ng.weights.optimizer_state_from_npz(p)
