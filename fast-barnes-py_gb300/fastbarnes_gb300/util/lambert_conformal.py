"""Lambert conformal conic projection (Snyder 1987), as used by the sphere path.

Mirrors fastbarnes/util/lambert_conformal.py: create_proj (:50-94) on the host,
to_map (:113-123) on the GPU.  A projection 'instance' is the tuple
(center_lon, n, n_inv, F, rho0).
"""
import ctypes

import numpy as np

from .. import _lib


def create_proj(center_lon, center_lat, lat1, lat2):
    """Projection constants (center_lon, n, n_inv, F, rho0) for the given
    center meridian / parallel and standard parallels lat1, lat2 [deg]."""
    p = (ctypes.c_double * 5)()
    _lib.lib().fb_lambert_create_proj(float(center_lon), float(center_lat), float(lat1), float(lat2), p)
    return tuple(p)


def to_map(geoc, mapc, center_lon, n, n_inv, F, rho0):
    """Maps the N x 2 lon/lat array geoc onto the Lambert map, writing the
    N x 2 map coordinates into mapc (and returning it), computed on the GPU.
    CUDA torch tensors are accepted for both arrays."""
    torch = _lib.torch_cuda()
    dev = geoc.device if isinstance(geoc, torch.Tensor) and geoc.is_cuda else \
        torch.device("cuda", torch.cuda.current_device())
    g = torch.as_tensor(geoc).to(device=dev, dtype=torch.float64).reshape(-1, 2).contiguous()
    m = torch.empty_like(g)
    proj = _lib.dvec([center_lon, n, n_inv, F, rho0])
    with torch.cuda.device(dev):
        _lib.check(_lib.lib().fb_lambert_to_map(g.data_ptr(), m.data_ptr(), g.shape[0], proj,
                                                _lib.stream_ptr(torch, dev)), "fb_lambert_to_map")
    if isinstance(mapc, torch.Tensor):
        mapc.copy_(m.reshape(mapc.shape))
    else:
        mapc[...] = m.cpu().numpy().reshape(np.shape(mapc))
    return mapc
