"""Seeded synthetic porous volumes of the benchmark workloads.

All generators return (SZ, SX, SY) uint8 arrays in the reference's input convention:
non-zero = solid, 0 = void (EuclideanDistanceComputer.cpp:167). The workloads:
  sphere_union   solid = union of spheres with uniform centres and radii (128^3, 300 spheres,
                 radii U[5,10]);
  grf            thresholded Gaussian random field: i.i.d. N(0,1), isotropic Gaussian blur,
                 void above the porosity quantile (512^3, sigma 3, porosity 0.65);
  spinodal       leveled-wave model: sum of cosines with |k| = 2 pi / wavelength, directions
                 uniform on the sphere, uniform phases (1024^3, 1000 waves, wavelength 48,
                 porosity 0.70);
  sphere_pack    spheres with uniform radii added until a solid fraction is reached
                 (batch sub-volumes).
Large sizes run on the GPU through torch; the quantile of grf/spinodal is taken from a
seeded sample of 2^24 voxels.
"""
import math

import numpy as np


def sphere_union(shape=(128, 128, 128), count=300, rmin=5.0, rmax=10.0, seed=1):
    """shape is (SZ, SX, SY). Centres uniform in the box (non-periodic)."""
    rng = np.random.default_rng(seed)
    sz, sx, sy = shape
    centres = rng.uniform(0, 1, size=(count, 3)) * np.array([sz, sx, sy])
    radii = rng.uniform(rmin, rmax, size=count)
    solid = np.zeros(shape, dtype=np.uint8)
    for (cz, cx, cy), r in zip(centres, radii):
        z0, z1 = max(0, int(math.floor(cz - r))), min(sz, int(math.ceil(cz + r)) + 1)
        x0, x1 = max(0, int(math.floor(cx - r))), min(sx, int(math.ceil(cx + r)) + 1)
        y0, y1 = max(0, int(math.floor(cy - r))), min(sy, int(math.ceil(cy + r)) + 1)
        if z0 >= z1 or x0 >= x1 or y0 >= y1:
            continue
        zz, xx, yy = np.ogrid[z0:z1, x0:x1, y0:y1]
        inside = (zz - cz) ** 2 + (xx - cx) ** 2 + (yy - cy) ** 2 <= r * r
        solid[z0:z1, x0:x1, y0:y1] |= inside.astype(np.uint8)
    return solid


def sphere_pack(shape, rmin=3.0, rmax=12.0, solid_fraction=0.40, seed=4):
    """Adds spheres (uniform centres and radii) until the solid fraction is reached."""
    rng = np.random.default_rng(seed)
    sz, sx, sy = shape
    solid = np.zeros(shape, dtype=np.uint8)
    total = solid.size
    filled = 0
    target = solid_fraction * total
    while filled < target:
        cz, cx, cy = rng.uniform(0, 1, 3) * np.array([sz, sx, sy])
        r = rng.uniform(rmin, rmax)
        z0, z1 = max(0, int(math.floor(cz - r))), min(sz, int(math.ceil(cz + r)) + 1)
        x0, x1 = max(0, int(math.floor(cx - r))), min(sx, int(math.ceil(cx + r)) + 1)
        y0, y1 = max(0, int(math.floor(cy - r))), min(sy, int(math.ceil(cy + r)) + 1)
        if z0 >= z1 or x0 >= x1 or y0 >= y1:
            continue
        zz, xx, yy = np.ogrid[z0:z1, x0:x1, y0:y1]
        inside = ((zz - cz) ** 2 + (xx - cx) ** 2 + (yy - cy) ** 2 <= r * r)
        block = solid[z0:z1, x0:x1, y0:y1]
        filled += int(np.count_nonzero(inside & (block == 0)))
        block |= inside.astype(np.uint8)
    return solid


def batch_shapes(count=256, lo=32, hi=192, seed=4):
    """Axis lengths drawn independently log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    return [tuple(int(round(math.exp(v))) for v in rng.uniform(math.log(lo), math.log(hi), 3))
            for _ in range(count)]


def _threshold_quantile(field_flat_sample, q):
    return float(np.quantile(field_flat_sample, q))


def grf(shape=(512, 512, 512), sigma=3.0, porosity=0.65, seed=2, device=None):
    """Thresholded Gaussian random field; void where the blurred field exceeds its
    (1 - porosity) quantile. Runs on `device` (a torch CUDA device) when given."""
    if device is None:
        from scipy import ndimage
        rng = np.random.default_rng(seed)
        f = rng.standard_normal(shape).astype(np.float32)
        f = ndimage.gaussian_filter(f, sigma, mode="reflect", truncate=4.0)
        t = np.quantile(f, 1.0 - porosity)
        return (f <= t).astype(np.uint8)
    import torch
    g = torch.Generator(device=device).manual_seed(seed)
    f = torch.randn(shape, generator=g, device=device, dtype=torch.float32)
    rad = int(4 * sigma + 0.5)
    xs = torch.arange(-rad, rad + 1, device=device, dtype=torch.float32)
    k = torch.exp(-0.5 * (xs / sigma) ** 2)
    k = (k / k.sum()).view(1, 1, -1)
    for axis in range(3):
        f = f.movedim(axis, -1).contiguous()
        s = f.shape
        n = s[-1]
        # reflect padding ("reflect" mode of scipy.ndimage: the edge sample is repeated)
        left = torch.arange(rad - 1, -1, -1, device=device).clamp(max=n - 1)
        right = torch.arange(n - 1, n - 1 - rad, -1, device=device).clamp(min=0)
        idx = torch.cat([left, torch.arange(n, device=device), right])
        flat = f.reshape(-1, n)
        out = torch.empty_like(flat)
        step = 1 << 15
        for r0 in range(0, flat.shape[0], step):
            blk = flat[r0:r0 + step].index_select(1, idx).unsqueeze(1)
            out[r0:r0 + step] = torch.nn.functional.conv1d(blk, k).squeeze(1)
        f = out.reshape(s).movedim(-1, axis)
    idx = torch.randint(0, f.numel(), (1 << 24,), generator=g, device=device)
    t = torch.quantile(f.reshape(-1)[idx].double(), 1.0 - porosity).float()
    return (f <= t).to(torch.uint8)


def grf_exact(shape=(512, 512, 512), sigma=3.0, porosity=0.65, seed=2):
    """Thresholded Gaussian random field computed in exact arithmetic, so that every machine
    builds the same volume bit for bit (the parity fixtures of the 512^3 workload are taken on
    one machine and checked on another). N(0,1) voxels are rounded to multiples of 1/256 and
    blurred with integer weights round(1024 exp(-k^2 / 2 sigma^2)), |k| <= round(4 sigma),
    along each axis (reflect mode, the edge sample repeated); every partial sum is an integer
    below 2^53, so float64 holds it exactly whatever the order of the additions. Solid where
    the field is at or below its k-th smallest value, k = floor((1 - porosity) * voxels)."""
    from scipy import ndimage
    rng = np.random.default_rng(seed)
    f = np.rint(rng.standard_normal(shape) * 256.0)
    rad = int(4 * sigma + 0.5)
    w = np.rint(1024.0 * np.exp(-0.5 * (np.arange(-rad, rad + 1) / sigma) ** 2))
    assert np.abs(f).max() * w.sum() ** 3 < 2.0 ** 53
    for axis in range(3):
        f = ndimage.correlate1d(f, w, axis=axis, mode="reflect")
    k = int((1.0 - porosity) * f.size)
    t = np.partition(f.reshape(-1), k)[k]
    return (f <= t).astype(np.uint8)


def spinodal(shape=(1024, 1024, 1024), waves=1000, wavelength=48.0, porosity=0.70, seed=3,
             device=None, chunk=16):
    """Leveled-wave monolith: f = sum_i cos(k_i . x + phi_i); void where f exceeds its
    (1 - porosity) quantile. Evaluated slab by slab as a complex matrix product
    f(z, x, y) = Re sum_i a_i(z) X_i(x) Y_i(y). Returns a torch uint8 tensor on `device`."""
    import torch
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((waves, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    kvec = v * (2.0 * math.pi / wavelength)
    phi = rng.uniform(0, 2 * math.pi, waves)
    sz, sx, sy = shape
    dev = device or "cuda"
    kz = torch.tensor(kvec[:, 0], device=dev, dtype=torch.float64)
    kx = torch.tensor(kvec[:, 1], device=dev, dtype=torch.float64)
    ky = torch.tensor(kvec[:, 2], device=dev, dtype=torch.float64)
    ph = torch.tensor(phi, device=dev, dtype=torch.float64)
    X = torch.exp(1j * kx[None, :] * torch.arange(sx, device=dev, dtype=torch.float64)[:, None])
    Y = torch.exp(1j * ky[:, None] * torch.arange(sy, device=dev, dtype=torch.float64)[None, :])
    X = X.to(torch.complex64)
    Y = Y.to(torch.complex64)
    out = torch.empty(shape, dtype=torch.float32, device=dev)
    zs = torch.arange(sz, device=dev, dtype=torch.float64)
    A = torch.exp(1j * (kz[None, :] * zs[:, None] + ph[None, :])).to(torch.complex64)  # (sz, waves)
    for z0 in range(0, sz, chunk):
        a = A[z0:z0 + chunk]                                  # (c, waves)
        lhs = a[:, None, :] * X[None, :, :]                   # (c, sx, waves)
        out[z0:z0 + chunk] = torch.matmul(lhs, Y).real        # (c, sx, sy)
    g = torch.Generator(device=dev).manual_seed(seed)
    idx = torch.randint(0, out.numel(), (1 << 24,), generator=g, device=dev)
    t = torch.quantile(out.reshape(-1)[idx].double(), 1.0 - porosity).float()
    return (out <= t).to(torch.uint8)


def sphere_pack_gpu(shape, ctx, rmin=3.0, rmax=12.0, solid_fraction=0.40, seed=4, classes=10,
                    device="cuda"):
    """Sphere pack for large volumes, generated on the GPU: a Boolean model whose sphere count
    gives the expected solid fraction, with radii uniform in [rmin, rmax] quantised to
    `classes` values. Each radius class is drawn as the voxels within r of its centres, using
    the squared distance transform of the centre points (pma_edt). Returns a (SZ, SX, SY)
    uint8 CUDA tensor, 1 = solid."""
    import torch
    from . import compute_euclidean_distances
    sz, sx, sy = shape
    n = sz * sx * sy
    radii = rmin + (np.arange(classes) + 0.5) * (rmax - rmin) / classes
    mean_volume = float(np.mean(4.0 / 3.0 * np.pi * radii ** 3))
    density = -math.log(1.0 - solid_fraction) / mean_volume  # centres per voxel
    rng = np.random.default_rng(seed)
    solid = torch.zeros(shape, dtype=torch.uint8, device=device)
    for r in radii:
        count = int(rng.poisson(density * n / classes))
        if count == 0:
            continue
        pts = torch.zeros(n, dtype=torch.uint8, device=device)
        pts[torch.from_numpy(rng.integers(0, n, count)).to(device)] = 1
        edt2, _, _ = compute_euclidean_distances(ctx, pts.view(shape))
        solid |= (edt2 <= int(r * r)).to(torch.uint8)
        del edt2, pts
    return solid
