"""Seeded synthetic rays in the shapes of the reference's workloads.

The reference renders Blender "lego" (800x800, focal 1111.111, near 2,
far 6; nerf/core/datasets.py:195-216, config.yaml:72) from cameras on a
radius-4 sphere that look at the origin (pose_utils.create_spherical_path,
pose_utils.py:770-840). That dataset is not available, so these generators
produce rays of the same geometry from a seed.
"""
import numpy as np


def _normalize(v):
    return v / (np.sqrt(np.sum(v ** 2, axis=-1, keepdims=True)) + 1e-8)


def sphere_rays(n, seed, radius=4.0, dir_sigma=0.05, near=2.0, far=6.0):
    """n rays with origins uniform on a sphere of `radius`, directions towards
    the centre perturbed by N(0, dir_sigma^2) per component, then normalised.
    Returns float32 (rays_o [n,3], rays_d [n,3], near [n,1], far [n,1])."""
    rng = np.random.default_rng(seed)
    nh = _normalize(rng.normal(size=(n, 3)))
    o = radius * nh
    d = _normalize(-nh + rng.normal(scale=dir_sigma, size=(n, 3)))
    return (o.astype(np.float32), d.astype(np.float32),
            np.full((n, 1), near, np.float32), np.full((n, 1), far, np.float32))


def look_at_pose(azimuth, inclination, radius=4.0):
    """Camera-to-world 4x4 pose on the sphere, camera z towards the origin,
    built as pose_utils.create_spherical_path does (pose_utils.py:798-830)."""
    p = radius * np.array([np.sin(inclination) * np.cos(azimuth),
                           np.sin(inclination) * np.sin(azimuth),
                           np.cos(inclination)])
    z = _normalize(-p)
    x = _normalize(np.array([-radius * np.sin(inclination) * np.sin(azimuth),
                             radius * np.sin(inclination) * np.cos(azimuth), 0.0]))
    y = _normalize(np.cross(z, x))
    pose = np.eye(4)
    pose[:3, 0], pose[:3, 1], pose[:3, 2], pose[:3, 3] = x, y, z, p
    return pose


def random_pose(seed, radius=4.0):
    rng = np.random.default_rng(seed)
    az = rng.uniform(0.0, 2.0 * np.pi)
    inc = np.arccos(rng.uniform(-0.9, 0.9))
    return look_at_pose(az, inc, radius)


def intrinsic(H=800, W=800, focal=1111.111):
    return np.array([[focal, 0.0, W / 2.0], [0.0, focal, H / 2.0], [0.0, 0.0, 1.0]])


def get_rays(H, W, K, c2w):
    """ray_utils.get_rays (ray_utils.py:6-51) in float64: pixel (u, v) ->
    ((u - cx)/fx, (v - cy)/fy, 1), rotated by c2w, normalised with EPS 1e-8;
    origin c2w[:3, 3]."""
    u, v = np.meshgrid(np.arange(W, dtype=np.float64), np.arange(H, dtype=np.float64), indexing="xy")
    dirs = np.stack([(u - K[0, 2]) / K[0, 0], (v - K[1, 2]) / K[1, 1], np.ones_like(u)], -1)
    d = _normalize(dirs.reshape(-1, 3) @ c2w[:3, :3].T)
    o = np.broadcast_to(c2w[:3, 3], d.shape)
    return o, d


def frame_rays(seed, H=800, W=800, focal=1111.111, radius=4.0, near=2.0, far=6.0):
    """All H*W rays of one pinhole frame from a random camera on the sphere.
    Returns float32 (rays_o, rays_d, near, far) as create_dataset_for_render
    casts them (base_dataset.py:846-851)."""
    o, d = get_rays(H, W, intrinsic(H, W, focal), random_pose(seed, radius))
    n = o.shape[0]
    return (np.ascontiguousarray(o, np.float32), d.astype(np.float32),
            np.full((n, 1), near, np.float32), np.full((n, 1), far, np.float32))


def sparse_scene_blob(seed, sigma_scale=4.0, sigma_bias=-0.5, max_freq_log2=None):
    """Parameters of a random-init NeRF network whose density is concentrated
    in sparse blobs: Glorot weights (the Keras default) with the sigma head's
    kernel scaled by `sigma_scale` and its bias set to `sigma_bias`. Used as
    both the coarse and the fine network (a trained NeRF's coarse and fine
    networks model the same scene), it gives a scene in which hierarchical
    sampling matters, unlike a plain random init whose density is noise.
    With `max_freq_log2` = m, the xyz encoding inputs of frequency 2^l pi,
    l >= m, are cut from dense_0 and from the dense_5 skip (a band-limited
    scene, like a real object whose extent is coarser than its detail)."""
    from .weights import glorot_blob, offsets
    blob = glorot_blob(seed)
    off = offsets()
    ko, bo, i, o = off["sigma"]
    blob[ko:ko + i * o] *= sigma_scale
    blob[bo] = sigma_bias
    if max_freq_log2 is not None:
        for layer, row0 in (("dense_0", 0), ("dense_5", 256)):
            ko, bo, i, o = off[layer]
            W = blob[ko:ko + i * o].reshape(i, o)
            for c in range(3):
                for l in range(max_freq_log2, 10):
                    W[row0 + 3 + c * 20 + 2 * l:row0 + 3 + c * 20 + 2 * l + 2, :] = 0.0
    return blob


def training_rays(seed, n_frames, rays_per_frame, H=800, W=800, focal=1111.111, near=2.0, far=6.0):
    """`rays_per_frame` random pixels from each of `n_frames` random cameras
    (the reference's sample-mode batches, base_dataset.py:555-621). Only the
    chosen pixels' rays are computed; they equal frame_rays' rows."""
    rng = np.random.default_rng(seed)
    K = intrinsic(H, W, focal)
    parts = [[], []]
    for f in range(n_frames):
        c2w = random_pose(seed * 1000 + f)
        idx = rng.choice(H * W, rays_per_frame, replace=False)
        u, v = (idx % W).astype(np.float64), (idx // W).astype(np.float64)
        dirs = np.stack([(u - K[0, 2]) / K[0, 0], (v - K[1, 2]) / K[1, 1], np.ones_like(u)], -1)
        d = _normalize(dirs @ c2w[:3, :3].T)
        parts[0].append(np.broadcast_to(c2w[:3, 3], d.shape).astype(np.float32))
        parts[1].append(d.astype(np.float32))
    o, d = np.concatenate(parts[0]), np.concatenate(parts[1])
    n = o.shape[0]
    return o, d, np.full((n, 1), near, np.float32), np.full((n, 1), far, np.float32)
