"""Persistent autotuner cache for the FdF kernel plans.

The autotuner times every compiled plan (pipeline depth, kernel variant) of
a likelihood's shape at finishInit and keeps the fastest, per (waves,
negative waves, rank, event-count class), in the process.  save() writes
those choices to a JSON file tagged with the device name, load() merges a
file back (refused for another device model), so that later processes take
the measured plans without timing runs."""
import ctypes as C

from . import _native as N


def save(path):
    N.call("pwa_autotune_cache_save", str(path).encode())


def load(path):
    N.call("pwa_autotune_cache_load", str(path).encode())


def clear():
    N.call("pwa_autotune_cache_clear")


def size():
    n = C.c_uint32()
    N.call("pwa_autotune_cache_size", C.byref(n))
    return n.value
