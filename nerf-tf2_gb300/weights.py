"""Parameters of one coarse or fine network as one flat float32 blob.

Layer order and shapes follow get_coarse_or_fine_model
(nerf/core/model.py:334-394); names follow its Keras layer names
("coarse/dense_0" ... "coarse/rgb"). Per layer the blob holds the Keras kernel
[in, out] row-major, then the bias [out]. Initialisation is the Keras Dense
default: GlorotUniform kernel, zero bias.
"""
import numpy as np

LAYERS = (
    ("dense_0", 63, 256), ("dense_1", 256, 256), ("dense_2", 256, 256),
    ("dense_3", 256, 256), ("dense_4", 256, 256), ("dense_5", 319, 256),
    ("dense_6", 256, 256), ("dense_7", 256, 256), ("sigma", 256, 1),
    ("dense_8", 256, 256), ("dense_9", 283, 128), ("rgb", 128, 3),
)
PARAM_COUNT = sum(i * o + o for _, i, o in LAYERS)  # 595,844


def offsets():
    """{name: (kernel_offset, bias_offset, in, out)} into the flat blob."""
    out, off = {}, 0
    for name, i, o in LAYERS:
        out[name] = (off, off + i * o, i, o)
        off += i * o + o
    return out


def glorot_blob(seed):
    """Flat float32 blob, Glorot-uniform kernels (limit sqrt(6/(in+out))),
    zero biases, drawn layer by layer from numpy's PCG64 with `seed`."""
    rng = np.random.default_rng(seed)
    parts = []
    for _, i, o in LAYERS:
        lim = np.sqrt(6.0 / (i + o))
        parts.append(rng.uniform(-lim, lim, size=(i, o)).astype(np.float32).reshape(-1))
        parts.append(np.zeros(o, np.float32))
    return np.concatenate(parts)


def to_dict(blob, model_name="coarse"):
    """Flat blob -> {"<model>/<layer>/kernel:0": array, ".../bias:0": array},
    the variable names Keras gives the reference's layers."""
    blob = np.asarray(blob)
    d = {}
    for name, (ko, bo, i, o) in offsets().items():
        d[f"{model_name}/{name}/kernel:0"] = blob[ko:ko + i * o].reshape(i, o)
        d[f"{model_name}/{name}/bias:0"] = blob[bo:bo + o]
    return d


def from_dict(d, model_name="coarse"):
    parts = []
    for name, i, o in LAYERS:
        parts.append(np.asarray(d[f"{model_name}/{name}/kernel:0"], np.float32).reshape(-1))
        parts.append(np.asarray(d[f"{model_name}/{name}/bias:0"], np.float32).reshape(-1))
    return np.concatenate(parts)


def from_keras_layers(layers, model_name="coarse"):
    """Weights read from a Keras weight file (h5.keras_layer_weights:
    [(layer name, [(weight name, array), ...]), ...]) ->
    {"<model>/<layer>/kernel:0": ..., ...}. As Keras's load_weights does for
    an HDF5 file (by topology, not by name), the file's layers that hold
    weights are matched in order to the network's (dense_0..7, sigma,
    dense_8, dense_9, rgb), each as [kernel, bias]; shapes must agree."""
    if len(layers) != len(LAYERS):
        raise ValueError(f"the file has {len(layers)} layers with weights, the network has {len(LAYERS)}")
    d = {}
    for (lname, ws), (name, i, o) in zip(layers, LAYERS):
        if len(ws) != 2:
            raise ValueError(f"layer {lname}: {len(ws)} weights, expected kernel and bias")
        (_, k), (_, b) = ws
        if tuple(k.shape) != (i, o) or tuple(b.shape) != (o,):
            raise ValueError(f"layer {lname}: shapes {tuple(k.shape)}, {tuple(b.shape)}; expected ({i}, {o}), ({o},)")
        d[f"{model_name}/{name}/kernel:0"] = np.asarray(k, np.float32)
        d[f"{model_name}/{name}/bias:0"] = np.asarray(b, np.float32)
    return d
