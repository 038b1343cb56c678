"""CORSIKA IACT photon bunches as the ray source of a trace.

``ACorsikaIACTFile`` mirrors the reference class (include/ACorsikaIACTFile.h,
src/ACorsikaIACTFile.cxx): Open a (gzip-compressed or plain) eventio file,
read its run header and telescope positions, ReadEvent(num), inspect the
bunches, and GetRayArray(telNo, arrayNo, z, refractiveIndex).  The eventio
stream is parsed by the native reader (rbg_corsika_*); the bunch-to-ray
expansion with the air-mass back-projection runs on the GPU
(rbg_bunches_to_rays), so a CORSIKA event goes straight into a device ray
batch for AOpticsManager.TraceNonSequential.
"""
from __future__ import annotations

import ctypes as C
import datetime
import gzip
import math
from typing import Dict, Optional

import numpy as np

from . import _native as N

BUNCH_FIELDS = ("x", "y", "zem", "time", "cx", "cy", "cz", "lambda", "photons")


class ACorsikaIACTRunHeader:
    """The 273 words of the CORSIKA run header (ACorsikaIACTRunHeader)."""

    def __init__(self, words: np.ndarray):
        self.words = words

    def GetRunNumber(self) -> int:
        return int(self.words[1])

    def GetDateOfBeginRun(self) -> datetime.date:
        yymmdd = int(self.words[2])
        y, md = divmod(yymmdd, 10000)
        mo, d = divmod(md, 100)
        return datetime.date(y + (1900 if y > 50 else 2000), mo, d)

    def GetVersionOfProgram(self) -> float:
        return float(self.words[3])

    def GetNumberOfObservationLevels(self) -> int:
        return int(self.words[4])

    def GetHeightOfLevel(self, i: int) -> float:
        return float(self.words[4 + i]) if 1 <= i <= 10 else math.nan

    def GetSlopeOfEnergySpectrum(self) -> float:
        return float(self.words[15])

    def GetLowerLimitOfEnergyRange(self) -> float:
        return float(self.words[16])

    def GetUpperLimitOfEnergyRange(self) -> float:
        return float(self.words[17])


class ACorsikaIACTEventHeader:
    """The 273 words of the CORSIKA event header (ACorsikaIACTEventHeader)."""

    def __init__(self, words: np.ndarray):
        self.words = words

    def GetEventNumber(self) -> int:
        return int(self.words[1])

    def GetParticleID(self) -> int:
        return int(self.words[2])

    def GetTotalEnergy(self) -> float:
        return float(self.words[3])

    def GetZenithAngle(self) -> float:
        return float(self.words[10])

    def GetAzimuthAngle(self) -> float:
        return float(self.words[11])

    def GetMinWavelength(self) -> float:
        return float(self.words[95])

    def GetMaxWavelength(self) -> float:
        return float(self.words[96])


class ACorsikaIACTFile:
    def __init__(self):
        self._h = None
        self._data = None
        self.fFileName = ""

    # -- Open / Close (src/ACorsikaIACTFile.cxx:191-257, 43-68) -------------------
    def Open(self, fname: str):
        with open(fname, "rb") as f:
            raw = f.read()
        if raw[:2] == b"\x1f\x8b":
            raw = gzip.decompress(raw)
        self.OpenBuffer(raw)
        self.fFileName = fname

    def OpenBuffer(self, data: bytes):
        self.Close()
        h = C.c_void_p()
        N.check(N.lib().rbg_corsika_open(data, len(data), C.byref(h)), "rbg_corsika_open")
        self._h = h
        self._data = data

    def Close(self):
        if self._h is not None:
            N.lib().rbg_corsika_close(self._h)
        self._h = None
        self.fFileName = ""

    def __del__(self):
        try:
            self.Close()
        except Exception:
            pass

    def IsOpen(self) -> bool:
        return self._h is not None

    def _need(self):
        if self._h is None:
            raise RuntimeError("ACorsikaIACTFile: no file is open")

    # -- headers and telescopes ------------------------------------------------------
    def GetRunHeader(self) -> ACorsikaIACTRunHeader:
        self._need()
        w = np.zeros(273, dtype=np.float32)
        N.check(N.lib().rbg_corsika_run_header(self._h, w.ctypes.data_as(C.POINTER(C.c_float))), "run header")
        return ACorsikaIACTRunHeader(w)

    def GetEventHeader(self) -> ACorsikaIACTEventHeader:
        self._need()
        w = np.zeros(273, dtype=np.float32)
        N.check(N.lib().rbg_corsika_event_header(self._h, w.ctypes.data_as(C.POINTER(C.c_float))), "event header")
        return ACorsikaIACTEventHeader(w)

    def GetInputCard(self):
        self._need()
        n = C.c_int32()
        need = N.lib().rbg_corsika_input_lines(self._h, None, 0, C.byref(n))
        buf = C.create_string_buffer(max(need, 1))
        N.lib().rbg_corsika_input_lines(self._h, buf, len(buf), C.byref(n))
        return buf.value.decode(errors="replace").splitlines()

    def _telescopes(self):
        self._need()
        n = C.c_int32()
        N.lib().rbg_corsika_telescopes(self._h, 0, C.byref(n), None, None, None, None)
        arrs = [np.zeros(max(n.value, 1)) for _ in range(4)]
        dp = C.POINTER(C.c_double)
        N.lib().rbg_corsika_telescopes(self._h, n.value, C.byref(n), *(a.ctypes.data_as(dp) for a in arrs))
        return n.value, arrs

    def GetNumberOfTelescopes(self) -> int:
        return self._telescopes()[0]

    def _tel(self, i, k):
        n, arrs = self._telescopes()
        return float(arrs[k][i]) if 0 <= i < n else math.nan

    def GetTelescopeX(self, i):
        return self._tel(i, 0)

    def GetTelescopeY(self, i):
        return self._tel(i, 1)

    def GetTelescopeZ(self, i):
        return self._tel(i, 2)

    def GetTelescopeR(self, i):
        return self._tel(i, 3)

    # -- events (src/ACorsikaIACTFile.cxx:264-489) -----------------------------------
    def ReadEvent(self, num: int) -> int:
        self._need()
        ev = C.c_int32(-1)
        N.check(N.lib().rbg_corsika_read_event(self._h, int(num), C.byref(ev)), "rbg_corsika_read_event")
        return ev.value

    def GetOffsets(self):
        """(time offset, x offsets, y offsets) of the current event's arrays."""
        self._need()
        n = C.c_int32()
        toff = C.c_double()
        N.check(N.lib().rbg_corsika_offsets(self._h, 0, C.byref(n), C.byref(toff), None, None), "offsets")
        x, y = np.zeros(max(n.value, 1)), np.zeros(max(n.value, 1))
        dp = C.POINTER(C.c_double)
        N.lib().rbg_corsika_offsets(self._h, n.value, C.byref(n), C.byref(toff), x.ctypes.data_as(dp),
                                    y.ctypes.data_as(dp))
        return toff.value, x[: n.value], y[: n.value]

    def GetBunches(self, telNo: int = -1, arrayNo: int = -1) -> Dict[str, np.ndarray]:
        """The current event's bunches (the reference's TTree "tree"), as
        float32 arrays plus int32 tel / array."""
        self._need()
        n = int(N.lib().rbg_corsika_bunch_count(self._h, telNo, arrayNo))
        out = {f: np.zeros(n, dtype=np.float32) for f in BUNCH_FIELDS}
        out["tel"] = np.zeros(n, dtype=np.int32)
        out["array"] = np.zeros(n, dtype=np.int32)
        b = N.Bunches()
        b.n = n
        fp, ip = C.POINTER(C.c_float), C.POINTER(C.c_int32)
        b.tel = out["tel"].ctypes.data_as(ip)
        b.array = out["array"].ctypes.data_as(ip)
        for f in BUNCH_FIELDS:
            setattr(b, "lambda_" if f == "lambda" else f, out[f].ctypes.data_as(fp))
        N.check(N.lib().rbg_corsika_get_bunches(self._h, telNo, arrayNo, C.byref(b)), "bunches")
        return out

    # -- rays (src/ACorsikaIACTFile.cxx:71-133) ---------------------------------------
    def GetDeviceRays(self, telNo: int, arrayNo: int, z: float, refractiveIndex: float = 1.0, seed: int = 0,
                      lambda_range: Optional[tuple] = None, device="cuda:0", stream=None):
        """Rays of one telescope and array as DEVICE tensors (x, y, z, t,
        dx, dy, dz, lam) for rbg_trace: the bunches are copied to the GPU
        once and expanded there.  lambda_range (nm) defaults to the event
        header's wavelength band."""
        import torch

        from .device import _ptr

        b = self.GetBunches(telNo, arrayNo)
        if lambda_range is None:
            h = self.GetEventHeader()
            lambda_range = (h.GetMinWavelength(), h.GetMaxWavelength())
        n = len(b["x"])
        dev = {f: torch.as_tensor(b[f]).to(device) for f in BUNCH_FIELDS}
        db = N.Bunches()
        db.n = n
        fp = C.POINTER(C.c_float)
        for f in BUNCH_FIELDS:
            setattr(db, "lambda_" if f == "lambda" else f, C.cast(_ptr(dev[f]), fp))
        ws = torch.empty(max(1, int(N.lib().rbg_bunches_workspace_bytes(n))), dtype=torch.uint8, device=device)
        st = (stream if stream is not None else torch.cuda.current_stream()).cuda_stream
        tel_z = self.GetTelescopeZ(telNo)
        total = C.c_int64()
        args = (float(z), float(tel_z), float(refractiveIndex), float(lambda_range[0]), float(lambda_range[1]),
                int(seed), _ptr(ws))
        N.check(N.lib().rbg_bunches_to_rays(C.byref(db), *args, None, 0, C.byref(total), C.c_void_p(st)),
                "rbg_bunches_to_rays")
        m = total.value
        rays = {f: torch.empty(max(m, 1), dtype=torch.float64, device=device)
                for f in ("x", "y", "z", "t", "dx", "dy", "dz", "lam")}
        dp = C.POINTER(C.c_double)
        rs = N.Rays(m, *(C.cast(_ptr(rays[f]), dp) for f in ("x", "y", "z", "t", "dx", "dy", "dz", "lam")))
        N.check(N.lib().rbg_bunches_to_rays(C.byref(db), *args, C.byref(rs), m, C.byref(total), C.c_void_p(st)),
                "rbg_bunches_to_rays")
        return {k: v[:m] for k, v in rays.items()}

    def GetRayArray(self, telNo: int, arrayNo: int, z: float, refractiveIndex: float = 1.0, seed: int = 0,
                    lambda_range: Optional[tuple] = None):
        """ACorsikaIACTFile::GetRayArray: an ARayArray (host) of the rays of
        one telescope and array, expanded on the GPU."""
        from .manager import ARayArray

        r = self.GetDeviceRays(telNo, arrayNo, z, refractiveIndex, seed, lambda_range)
        h = {k: v.cpu().numpy() for k, v in r.items()}
        return ARayArray.from_arrays(h["x"], h["y"], h["z"], h["dx"], h["dy"], h["dz"], h["lam"], t=h["t"])
