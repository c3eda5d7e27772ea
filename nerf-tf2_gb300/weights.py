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
    {"<model>/<layer>/kernel:0": ..., ...}.

    Keras's load_weights pairs an HDF5 file's layers with the network's by
    position in model.layers, which for a functional model is the graph-depth
    order of the network that wrote the file (dense_0..7, dense_8, dense_9,
    rgb, sigma for get_coarse_or_fine_model, not the order of its source).
    The reference names every layer (model.py:366-387: "<model>/dense_i",
    "<model>/sigma", "<model>/rgb"), so the file's layers are matched here by
    that name, which gives the same pairing for a file the reference wrote
    and does not depend on the order of layer_names. Each layer holds
    [kernel, bias] with the network's shapes; the file must hold every layer
    of the network and no other layer with weights."""
    if len(layers) != len(LAYERS):
        raise ValueError(f"the file has {len(layers)} layers with weights, the network has {len(LAYERS)}")
    by_name = {}
    for lname, ws in layers:
        short = lname.rsplit("/", 1)[-1]
        if short in by_name:
            raise ValueError(f"layer {lname}: the file names layer {short!r} twice")
        by_name[short] = (lname, ws)
    d = {}
    for name, i, o in LAYERS:
        if name not in by_name:
            raise ValueError(f"the file has no layer {model_name}/{name} (its layers: {sorted(by_name)})")
        lname, ws = by_name[name]
        if len(ws) != 2:
            raise ValueError(f"layer {lname}: {len(ws)} weights, expected kernel and bias")
        (_, k), (_, b) = ws
        if tuple(k.shape) != (i, o) or tuple(b.shape) != (o,):
            raise ValueError(f"layer {lname}: shapes {tuple(k.shape)}, {tuple(b.shape)}; expected ({i}, {o}), ({o},)")
        d[f"{model_name}/{name}/kernel:0"] = np.asarray(k, np.float32)
        d[f"{model_name}/{name}/bias:0"] = np.asarray(b, np.float32)
    return d


def optimizer_state_from_npz(path, model_names=("coarse", "fine")):
    """The Adam state the reference saves as <tag>_optimizer.npz
    (nerf/core/ops.py:110-120 writes optimizer.variables() with np.savez,
    plus "names" for their order; nerf/core/model.py:246-276 reads it back).

    Keras names Adam's variables "<optimizer>/iter:0" (the step count),
    "<optimizer>/beta_1:0" etc. (hyperparameters) and, per trainable
    variable "<model>/<layer>/kernel:0", the slots
    "<optimizer>/<model>/<layer>/kernel/m:0" and ".../v:0". The reference
    checks that the saved names equal those of the optimizer it rebuilt, in
    order; here the slots are matched by name instead, onto this package's
    flat parameter layout, and every slot of every layer must be present
    with its variable's shape. Saved beta_1/beta_2 must be Keras's defaults
    (0.9, 0.999), the values the reference's Adam uses (model.py:413-418).

    Returns {"step": int, "m": {model: blob}, "v": {model: blob}} with
    float32 blobs of PARAM_COUNT values."""
    data = np.load(path, allow_pickle=False)
    names = [str(x) for x in data["names"]]
    step = None
    slots = {}
    for full in names:
        base = full[:-2] if full.endswith(":0") else full
        if base.endswith("/iter") or base == "iter":
            step = int(np.asarray(data[full]).reshape(()))
            continue
        leaf = base.rsplit("/", 1)[-1]
        if leaf in ("beta_1", "beta_2"):
            want = 0.9 if leaf == "beta_1" else 0.999
            if not np.isclose(float(np.asarray(data[full]).reshape(())), want, rtol=0, atol=1e-7):
                raise ValueError(f"{full}: saved Adam {leaf} differs from the reference's {want}")
            continue
        if leaf not in ("m", "v"):
            continue  # decay, learning_rate: the schedule is recomputed from the step
        parts = base.split("/")
        if len(parts) < 4 or parts[-2] not in ("kernel", "bias"):
            raise ValueError(f"{full}: not a slot of a kernel or bias variable")
        key = (parts[-4], parts[-3], parts[-2], leaf)  # model, layer, kernel|bias, m|v
        if key in slots:
            raise ValueError(f"{full}: slot saved twice")
        slots[key] = np.asarray(data[full], np.float32)
    if step is None:
        raise ValueError(f"{path}: no iteration count (…/iter:0) among the saved names")
    out = {"step": step, "m": {}, "v": {}}
    for model in model_names:
        for slot in ("m", "v"):
            parts = []
            for name, i, o in LAYERS:
                for kind, shape in (("kernel", (i, o)), ("bias", (o,))):
                    a = slots.get((model, name, kind, slot))
                    if a is None:
                        raise ValueError(f"{path}: no Adam slot {slot} for {model}/{name}/{kind}")
                    if tuple(a.shape) != shape:
                        raise ValueError(f"{model}/{name}/{kind}/{slot}: shape {tuple(a.shape)}, expected {shape}")
                    parts.append(a.reshape(-1))
            out[slot][model] = np.concatenate(parts)
    return out
