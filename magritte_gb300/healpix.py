"""HEALPix RING-scheme pixel centres and Magritte's uniform-ray rotation.

The reference builds its ray directions with ``healpy.pixelfunc.pix2vec`` and then
rotates them so that ray 0 points along ``first_ray`` (magritte/setup.py:174-223,
rotation helper :101-122).  healpy is not a dependency here, so the pixel centres
are computed from the published RING-scheme formulae (Gorski et al. 2005, ApJ 622,
759, section 4): north polar cap, equatorial belt, south polar cap.  In RING order
pixel ``i`` and pixel ``npix-1-i`` are antipodal, which is what the solver's
ray-pair loop relies on (rays ``r`` and ``antipod[r]``).
"""
import math

import numpy as np


def nside2npix(nside: int) -> int:
    return 12 * nside * nside


def npix2nside(npix: int) -> int:
    nside = int(round(math.sqrt(npix / 12)))
    if 12 * nside * nside != npix:
        raise ValueError(f"{npix} is not a valid HEALPix pixel count")
    return nside


def pix2vec_ring(nside: int, pixels=None) -> np.ndarray:
    """Unit vectors (npix, 3) of the RING-scheme pixel centres."""
    npix = nside2npix(nside)
    if pixels is None:
        pixels = range(npix)
    ncap = 2 * nside * (nside - 1)
    out = []
    for p in pixels:
        if p < ncap:  # north polar cap
            iring = int(0.5 * (1 + math.isqrt(1 + 2 * p)))
            # guard the integer square root at ring boundaries
            while 2 * iring * (iring - 1) > p:
                iring -= 1
            while 2 * (iring + 1) * iring <= p:
                iring += 1
            iphi = p + 1 - 2 * iring * (iring - 1)
            z = 1.0 - iring * iring / (3.0 * nside * nside)
            phi = (iphi - 0.5) * (0.5 * math.pi) / iring
        elif p < npix - ncap:  # equatorial belt
            ip = p - ncap
            iring = ip // (4 * nside) + nside
            iphi = ip % (4 * nside) + 1
            fodd = 1.0 if ((iring + nside) & 1) else 0.5
            z = (2 * nside - iring) / (1.5 * nside)
            phi = (iphi - fodd) * (0.5 * math.pi) / nside
        else:  # south polar cap
            ip = npix - p
            iring = int(0.5 * (1 + math.isqrt(2 * ip - 1)))
            while 2 * iring * (iring - 1) >= ip:
                iring -= 1
            while 2 * (iring + 1) * iring < ip:
                iring += 1
            iphi = 4 * iring + 1 - (ip - 2 * iring * (iring - 1))
            z = -1.0 + iring * iring / (3.0 * nside * nside)
            phi = (iphi - 0.5) * (0.5 * math.pi) / iring
        s = math.sqrt(max(0.0, (1.0 - z) * (1.0 + z)))
        out.append((s * math.cos(phi), s * math.sin(phi), z))
    return np.array(out, dtype=np.float64)


def rotation_matrix(n) -> np.ndarray:
    """Orthonormal frame whose first column is ``n`` (magritte/setup.py:101-122)."""
    nx = np.array([1.0, 0.0, 0.0])
    ny = np.array([0.0, 1.0, 0.0])
    n1 = np.array(n, dtype=np.float64)
    n1 = n1 / np.linalg.norm(n1)
    if np.linalg.norm(n1 - nx) < 1.0e-6:
        n2 = np.cross(ny, n1)
    else:
        n2 = np.cross(nx, n1)
    n2 = n2 / np.linalg.norm(n2)
    n3 = np.cross(n2, n1)
    n3 = n3 / np.linalg.norm(n3)
    return np.array([n1, n2, n3]).T


def uniform_rays(nrays: int, first_ray=(1.0, 0.0, 0.0)):
    """Directions and weights as ``set_uniform_rays`` produces them in 3D
    (magritte/setup.py:174-223): HEALPix pixel centres rotated so that ray 0 is
    ``first_ray``; every weight is 1/nrays."""
    direction = pix2vec_ring(npix2nside(nrays))
    R1 = rotation_matrix(direction[0])
    R2 = rotation_matrix(np.asarray(first_ray, dtype=np.float64))
    R = R2 @ np.linalg.inv(R1)
    direction = direction @ R.T
    weight = np.full(nrays, 1.0 / nrays)
    return direction, weight


def antipodes(direction: np.ndarray, tol: float = 1.0e-9) -> np.ndarray:
    """Antipode index per ray (src/model/geometry/rays/rays.cpp:53-60): the last r2
    with |d[r1] + d[r2]|^2 < tol."""
    n = direction.shape[0]
    s = direction[:, None, :] + direction[None, :, :]
    d2 = np.einsum("ijk,ijk->ij", s, s)
    out = np.zeros(n, dtype=np.uint32)
    for r1 in range(n):
        hits = np.nonzero(d2[r1] < tol)[0]
        if len(hits) == 0:
            raise ValueError(f"ray {r1} has no antipode")
        out[r1] = hits[-1]
    return out
