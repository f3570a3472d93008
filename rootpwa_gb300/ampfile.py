"""Raw amplitude files: the decay amplitudes of one event file for a set of
waves plus the event file's binning variables, in one flat file laid out for
sequential reads into device memory.

They stand in for the reference's per-wave ROOT trees of amplitudeTreeLeaf
objects (storageFormats/amplitudeTreeLeaf.h:51-118, read by
pwaLikelihood::addAmplitude, partialWaveFit/pwaLikelihood.cc:1110-1288) and
for the binning variables that setOnTheFlyBinning reads from the event
metadata (pwaLikelihood.cc:1391-1440).  Layout (little-endian):

    magic "RPWAAMP\\0" | u32 version 1 | u32 W | u32 V | u32 0 | u64 N |
    u64 data offset (multiple of 4096) | W wave names, V variable names
    (u16 length + bytes) | zero padding | W rows of N complex64 |
    V rows of N float64

writeAmplitudeFile and ampFileInfo go through the native library;
readAmplitudeFile is a numpy memory-map of the same layout for inspection.
Loading into a likelihood is pwaLikelihood.loadAmplitudeFiles."""
import ctypes as C

import numpy as np

from . import _native as N

_MAGIC = b"RPWAAMP\x00"


def _cstrs(names):
    enc = [n.encode() for n in names]
    return (C.c_char_p * max(1, len(enc)))(*enc)


def writeAmplitudeFile(path, waveNames, amps, binVars=None):
    """amps: [W][N] complex (stored as complex64); binVars: {name: [N]}."""
    a = np.ascontiguousarray(np.asarray(amps), dtype=np.complex64)
    if a.ndim != 2 or a.shape[0] != len(waveNames):
        raise ValueError("amps must be [nWaves][nEvents]")
    n = a.shape[1]
    binVars = binVars or {}
    vn = list(binVars)
    v = np.ascontiguousarray(np.stack([np.asarray(binVars[k], dtype=np.float64) for k in vn])) if vn else None
    if v is not None and v.shape[1] != n:
        raise ValueError("binning variables must have one value per event")
    N.call("pwa_ampfile_write", str(path).encode(), len(waveNames), _cstrs(waveNames), n,
           C.c_void_p(a.ctypes.data), len(vn), _cstrs(vn),
           v.ctypes.data_as(C.POINTER(C.c_double)) if v is not None else None)


def ampFileInfo(path):
    """(wave names, number of events, binning variable names)."""
    w, n, v = C.c_uint32(), C.c_uint64(), C.c_uint32()
    p = str(path).encode()
    N.call("pwa_ampfile_info", p, C.byref(w), C.byref(n), C.byref(v))
    buf = C.create_string_buffer(65536)
    waves, vars_ = [], []
    for k in range(w.value):
        N.call("pwa_ampfile_name", p, 0, k, buf, len(buf))
        waves.append(buf.value.decode())
    for k in range(v.value):
        N.call("pwa_ampfile_name", p, 1, k, buf, len(buf))
        vars_.append(buf.value.decode())
    return waves, n.value, vars_


def readAmplitudeFile(path):
    """(wave names, amps [W][N] complex64 memmap, {variable: [N] float64 memmap})."""
    with open(path, "rb") as f:
        head = f.read(40)
        if len(head) < 40 or head[:8] != _MAGIC:
            raise ValueError("%s is not an amplitude file" % path)
        version, W, V, _zero = np.frombuffer(head, dtype="<u4", count=4, offset=8)
        n, off = np.frombuffer(head, dtype="<u8", count=2, offset=24)
        if version != 1:
            raise ValueError("unsupported amplitude file version %d" % version)
        table = f.read(int(off) - 40)
    names, pos = [], 0
    for _ in range(int(W) + int(V)):
        ln = int(np.frombuffer(table, dtype="<u2", count=1, offset=pos)[0])
        names.append(table[pos + 2:pos + 2 + ln].decode())
        pos += 2 + ln
    W, V, n, off = int(W), int(V), int(n), int(off)
    amps = np.memmap(path, dtype="<c8", mode="r", offset=off, shape=(W, n)) if W and n else np.zeros((W, n), np.complex64)
    vars_ = {}
    if V and n:
        vm = np.memmap(path, dtype="<f8", mode="r", offset=off + 8 * W * n, shape=(V, n))
        vars_ = {names[W + k]: vm[k] for k in range(V)}
    return names[:W], amps, vars_
