"""Source fields on the device (mirror of optics-core ``sources::gaussian``,
src/sources.rs:259-296, and ``BandField::plane_wave`` / ``uniform``,
src/field.rs:315-386): torch tensors (ny, nx) on ``cuda``, complex128 or
complex64, evaluated per sample in FP64."""

from . import _ffi


def _out(nx, ny, dtype):
    import torch
    t = torch.empty((ny, nx), dtype=dtype, device="cuda")
    code = _ffi.C128 if dtype == torch.complex128 else _ffi.C64
    return t, code


def _sptr():
    from .inverse import _stream_handle
    return _stream_handle()


def gaussian(w0, amplitude, center, z, lam, nx, ny, dx, dy, dtype=None):
    """q-form Gaussian beam at distance z from its waist w0, centred at `center`."""
    import torch
    t, code = _out(nx, ny, dtype or torch.complex128)
    _ffi.check(_ffi.lib().osgpu_source_gaussian_device(
        t.data_ptr(), code, _ffi.Grid(nx, ny, dx, dy, lam), w0, amplitude, center[0], center[1],
        z, _sptr()))
    return t


def plane_wave(theta_x, theta_y, amplitude, nx, ny, dx, dy, lam, dtype=None):
    import torch
    t, code = _out(nx, ny, dtype or torch.complex128)
    _ffi.check(_ffi.lib().osgpu_source_plane_wave_device(
        t.data_ptr(), code, _ffi.Grid(nx, ny, dx, dy, lam), theta_x, theta_y, amplitude, _sptr()))
    return t


def uniform(amplitude, phase, nx, ny, dx, dy, lam, dtype=None):
    import torch
    t, code = _out(nx, ny, dtype or torch.complex128)
    _ffi.check(_ffi.lib().osgpu_source_uniform_device(
        t.data_ptr(), code, _ffi.Grid(nx, ny, dx, dy, lam), amplitude, phase, _sptr()))
    return t
