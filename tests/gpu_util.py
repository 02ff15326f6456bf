"""Helpers shared by the GPU parity tests."""
import numpy as np

STATE = ("u", "v", "w", "p", "S", "T", "Yo", "Yf", "Ys", "Ya", "Yp", "Yc", "Yw", "Yco", "Yai", "nu", "Pb", "Q", "Qr",
         "hrr", "massSrc")


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    d = np.linalg.norm(a - b)
    return d / nb if nb > 0 else d


def copy_state(src, dst, fields=STATE):
    for f in fields:
        dst.set(f, src.get(f))
    dst.set("lit", src.get("lit"))
    sc = src.scalars() if hasattr(src, "scalars") else None
    return sc
