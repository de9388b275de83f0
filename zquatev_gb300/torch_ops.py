"""torch custom operators over the device entry points.

``torch.ops.zquatev_gb300.zquatev(h_left)`` is ts::zquatev (reference
zquatev.h:54) for tensors that already live on the GPU: ``h_left`` is the
(n2, n) complex128 CUDA tensor [A; B] (A Hermitian, B complex antisymmetric:
the left half of H = (A -B*; B A*), which is all the reference reads). It
returns ``(eig, v)``: the n ascending eigenvalues (float64) and the (n2, n2)
eigenvectors in the (U -V*; V U*) layout, column j of ``v`` belonging to
``eig[j % n]``. The solve runs through ``zquatev_device`` (the drop-in's path
policy, refined from n = 48 up) on torch's current stream, without host
synchronisation. ``torch.ops.zquatev_gb300.eigvalsh(h_left)`` returns the
eigenvalues only (``zquatev_values_device``).

The operators are registered for CUDA only (a CPU tensor raises: there is no
CPU fallback) and have fake implementations, so they trace under FakeTensor /
meta tensors. They define no gradient.
"""
from __future__ import annotations

import torch

from . import _lib


def _column_major_work(h_left: torch.Tensor) -> torch.Tensor:
    """(n2, n2) tensor whose memory is the column-major n2 x n2 array D with
    [A; B] in its left half (row j of the tensor = column j of D)."""
    n2, n = h_left.shape
    work = torch.empty((n2, n2), dtype=torch.complex128, device=h_left.device)
    work[:n].copy_(h_left.T)
    return work


def _check(h_left: torch.Tensor) -> None:
    if h_left.dtype != torch.complex128 or h_left.dim() != 2 or h_left.shape[0] != 2 * h_left.shape[1]:
        raise ValueError("h_left must be an (n2, n2/2) complex128 tensor holding [A; B]")


@torch.library.custom_op("zquatev_gb300::zquatev", mutates_args=(), device_types="cuda")
def zquatev(h_left: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    _check(h_left)
    n2, n = h_left.shape
    work = _column_major_work(h_left)
    deig = torch.empty(max(n2, 1), dtype=torch.float64, device=h_left.device)
    st = torch.cuda.current_stream(h_left.device).cuda_stream
    with torch.cuda.device(h_left.device):
        _lib.check(_lib.load().zquatev_device(n2, work.data_ptr(), n2, deig.data_ptr(), st), "zquatev_device")
    return deig[:n].clone(), work.T.contiguous()


@zquatev.register_fake
def _(h_left):
    _check(h_left)
    n2, n = h_left.shape
    return h_left.new_empty((n,), dtype=torch.float64), h_left.new_empty((n2, n2))


@torch.library.custom_op("zquatev_gb300::eigvalsh", mutates_args=(), device_types="cuda")
def eigvalsh(h_left: torch.Tensor) -> torch.Tensor:
    _check(h_left)
    n2, n = h_left.shape
    work = _column_major_work(h_left)
    deig = torch.empty(max(n2, 1), dtype=torch.float64, device=h_left.device)
    st = torch.cuda.current_stream(h_left.device).cuda_stream
    with torch.cuda.device(h_left.device):
        _lib.check(_lib.load().zquatev_values_device(n2, work.data_ptr(), n2, deig.data_ptr(), st),
                   "zquatev_values_device")
    return deig[:n].clone()


@eigvalsh.register_fake
def _(h_left):
    _check(h_left)
    return h_left.new_empty((h_left.shape[1],), dtype=torch.float64)
