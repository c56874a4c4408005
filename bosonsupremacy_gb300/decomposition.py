"""Drop-in for get_decomposition.py: the pure quantum part of the covariance.

    python -m bosonsupremacy_gb300.decomposition --dir ROOT/

Same flag and files as get_decomposition.py:6-30: reads ROOT/cov.npy, writes
ROOT/sq_cov.npy, and does nothing when sq_cov.npy already exists (:12-14).
The SDP (get_decomposition.py:22-27)

    minimise tr X  s.t.  [[X, Omega], [-Omega, X]] >= 0,  cov - X >= 0

is solved on the GPU by bsg_cov_decomposition (a primal-dual interior-point
method in FP64); there is no CPU path.
"""
from __future__ import annotations

import argparse
import ctypes
import os

import numpy as np
import torch

from . import _lib


def decompose(cov, tol: float = 1e-10, max_iter: int = 100, device: int = 0, handle=None):
    """(sq_cov, info) for a 2M x 2M covariance (xxpp): sq_cov float64 numpy,
    info = {iterations, rel_gap, primal_res, dual_res, primal_obj, dual_obj}.
    Raises when the solver does not reach `tol` within `max_iter` iterations."""
    cov = np.asarray(cov, dtype=np.float64)
    if cov.ndim != 2 or cov.shape[0] != cov.shape[1] or cov.shape[0] % 2:
        raise ValueError("cov must be a square 2M x 2M matrix")
    M = cov.shape[0] // 2
    dev = torch.device("cuda", device)
    c = torch.as_tensor(cov).to(dev).contiguous()
    out = torch.empty_like(c)
    info = (ctypes.c_double * 6)()
    h = handle if handle is not None else _lib.Handle.get(device)
    _lib.check(_lib.load().bsg_cov_decomposition(h.h, c.data_ptr(), M, out.data_ptr(), float(tol), int(max_iter),
                                                 info, _lib.stream_ptr()),
               "bsg_cov_decomposition")
    keys = ("iterations", "rel_gap", "primal_res", "dual_res", "primal_obj", "dual_obj")
    meta = {k: float(v) for k, v in zip(keys, info)}
    meta["iterations"] = int(meta["iterations"])
    return out.cpu().numpy(), meta


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--dir", type=str, help="Experiment directory.")
    p.add_argument("--tol", type=float, default=1e-10)
    p.add_argument("--max-iter", type=int, default=100)
    args = p.parse_args(argv)
    rootdir = args.dir
    if os.path.isfile(rootdir + "sq_cov.npy"):
        print("Decomposition results already available.")
        return
    cov = np.load(rootdir + "cov.npy")
    sq_cov, meta = decompose(cov, tol=args.tol, max_iter=args.max_iter)
    print(f"{meta['iterations']} iterations, relative gap {meta['rel_gap']:.2e}")
    np.save(rootdir + "sq_cov.npy", sq_cov)


if __name__ == "__main__":
    main()
