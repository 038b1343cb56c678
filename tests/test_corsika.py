"""CORSIKA IACT ingestion: the eventio reader against what the reference's
own reader (src/bernlohr, compiled into oracle/_ref) reads from the
muon_ring4 event of tutorials/CORSIKA.C (tests/golden, made by
tests/golden/make_fixtures.py); synthetic streams for the compact bunch
format, per-telescope array blocks and malformed input; and, on the GPU,
the bunch-to-ray expansion of ACorsikaIACTFile::GetRayArray against its
oracle restatement, then a trace of the event."""
import ctypes as C
import gzip
import os
import struct

import numpy as np
import pytest

import oracle_ref
from robast_gb300 import _native as N
from robast_gb300 import configs
from robast_gb300.corsika import ACorsikaIACTFile

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "muon_ring4.corsika.gz")
GOLDEN = np.load(os.path.join(HERE, "golden", "corsika_muon_ring4.npz"))
SYNC = 0xD41F8A37


@pytest.fixture
def event():
    f = ACorsikaIACTFile()
    f.Open(FIXTURE)
    assert f.ReadEvent(1) == 1
    return f


def test_run_header_telescopes_and_input_card():
    f = ACorsikaIACTFile()
    f.Open(FIXTURE)
    rh = f.GetRunHeader()
    np.testing.assert_array_equal(rh.words[1:], GOLDEN["runh"][1:])
    assert rh.GetRunNumber() == 27
    assert rh.GetDateOfBeginRun().isoformat() == "2015-11-09"
    assert rh.GetVersionOfProgram() == pytest.approx(7.4005, abs=1e-4)
    assert rh.GetNumberOfObservationLevels() == 1
    assert rh.GetHeightOfLevel(1) == pytest.approx(200000.0)
    assert len(f.GetInputCard()) == int(GOLDEN["input_lines"])
    tel = GOLDEN["tel"]
    assert f.GetNumberOfTelescopes() == len(tel)
    for i, (x, y, z, r) in enumerate(tel):
        assert (f.GetTelescopeX(i), f.GetTelescopeY(i), f.GetTelescopeZ(i), f.GetTelescopeR(i)) == (x, y, z, r)
    assert np.isnan(f.GetTelescopeZ(len(tel)))


def test_event_header_offsets_and_bunches(event):
    eh = event.GetEventHeader()
    np.testing.assert_array_equal(eh.words[1:], GOLDEN["evth"][1:])
    assert eh.GetEventNumber() == 1
    toff, xo, yo = event.GetOffsets()
    assert toff == pytest.approx(float(GOLDEN["time_offset"]), rel=1e-7)
    np.testing.assert_array_equal(np.stack([xo, yo], axis=1), GOLDEN["offsets"])
    b = event.GetBunches()
    g = GOLDEN["bunch"]  # x, y, cx, cy, ctime, zem, photons, lambda
    assert len(b["x"]) == len(g) == 2842
    for k, name in enumerate(("x", "y", "cx", "cy", "time", "zem", "photons", "lambda")):
        np.testing.assert_array_equal(b[name], g[:, k], err_msg=name)
    np.testing.assert_array_equal(b["tel"], GOLDEN["bunch_tel"])
    np.testing.assert_array_equal(b["array"], GOLDEN["bunch_array"])
    # cz as ACorsikaIACTFile::ReadEvent computes it (squares in float)
    cz = (-np.sqrt(1.0 - (g[:, 2] * g[:, 2]).astype(np.float64) - (g[:, 3] * g[:, 3]).astype(np.float64)))
    np.testing.assert_array_equal(b["cz"], cz.astype(np.float32))
    assert len(event.GetBunches(0, 0)["x"]) == 2842 and len(event.GetBunches(1, 0)["x"]) == 0
    # re-reading the current event is a no-op; there is no event 2
    assert event.ReadEvent(1) == 1
    assert event.ReadEvent(2) == -1


# ---- synthetic streams -----------------------------------------------------
def _item(typ, ident, payload, version=0, sync=False, only_sub=False):
    head = struct.pack("<IiI", typ | (version << 20), ident, len(payload) | (0x40000000 if only_sub else 0))
    return (struct.pack("<I", SYNC) if sync else b"") + head + payload


def _header_block(typ, words):
    return _item(typ, 0, struct.pack("<ii", len(words), 0) + struct.pack(f"<{len(words) - 1}f", *words[1:]), sync=True)


def _stream(photon_blocks, head_end=False):
    runh = [0.0] * 273
    runh[1], runh[2], runh[3] = 5, 240101, 7.7
    evth = [0.0] * 273
    evth[1], evth[95], evth[96] = 1, 300, 600
    s = _header_block(1200, runh)
    s += _item(1212, 0, struct.pack("<i", 1) + struct.pack("<h", 4) + b"RUNN", sync=True)
    s += _item(1201, 0, struct.pack("<i", 2) + struct.pack("<8f", 0, 500, 0, 0, 1000, 1200, 600, 600), sync=True)
    s += _header_block(1202, evth)
    s += _item(1203, 0, struct.pack("<if", 1, 7.0) + struct.pack("<2f", 0.0, 0.0), sync=True)
    if head_end:
        s += _item(1213, 0, b"", sync=True)
        for blk in photon_blocks:
            s += _item(1205, 0, blk[1], version=blk[0], sync=True)
        s += _item(1214, 0, b"", sync=True)
    else:
        subs = b"".join(_item(1205, 0, blk[1], version=blk[0]) for blk in photon_blocks)
        s += _item(1204, 0, subs, sync=True, only_sub=True)
    s += _header_block(1209, [0.0] * 273)
    return s


def _compact(tel, shorts):
    body = struct.pack("<hhfi", 0, tel, 0.0, len(shorts)) + b"".join(struct.pack("<8h", *r) for r in shorts)
    return (1000, body)


def _long(tel, rows):
    body = struct.pack("<hhfi", 0, tel, 0.0, len(rows)) + b"".join(struct.pack("<8f", *r) for r in rows)
    return (0, body)


@pytest.mark.parametrize("head_end", [False, True])
def test_compact_and_long_bunch_formats(head_end):
    rows = [(123, -45, 3000, -1500, 77, 3000, 250, 0), (-7, 9, 31000, -31000, -5, 0, 1, 420)]
    longs = [(1.5, -2.5, 0.01, -0.02, 3.25, 8e5, 2.5, 0.0)]
    f = ACorsikaIACTFile()
    f.OpenBuffer(_stream([_compact(0, rows), _long(1, longs)], head_end))
    assert f.GetRunHeader().GetRunNumber() == 5 and f.GetInputCard() == ["RUNN"]
    assert f.GetNumberOfTelescopes() == 2 and f.GetTelescopeZ(1) == 1200
    assert f.ReadEvent(1) == 1
    b = f.GetBunches(0)
    np.testing.assert_array_equal(b["x"], np.float32([12.3, -0.7]))
    np.testing.assert_array_equal(b["y"], np.float32([-4.5, 0.9]))
    np.testing.assert_array_equal(b["cx"], np.float32([0.1, 1.0]))  # clamped to [-1, 1]
    np.testing.assert_array_equal(b["cy"], np.float32([-0.05, -1.0]))
    np.testing.assert_array_equal(b["time"], np.float32([7.7, -0.5]))
    np.testing.assert_array_equal(b["zem"], np.float32([10.0 ** 3.0, 1.0]))
    np.testing.assert_array_equal(b["photons"], np.float32([2.5, 0.01]))
    np.testing.assert_array_equal(b["lambda"], np.float32([0, 420]))
    bl = f.GetBunches(1)
    np.testing.assert_array_equal(np.stack([bl[k] for k in ("x", "y", "cx", "cy", "time", "zem", "photons",
                                                             "lambda")], axis=1), np.float32(longs))


def test_malformed_streams_are_rejected_not_read_out_of_bounds():
    good = _stream([_long(0, [(1, 2, 0.1, 0.1, 0, 1e5, 1, 400)] * 3)])
    for cut in (3, 17, 40, 1100, len(good) - 40):
        f = ACorsikaIACTFile()
        try:
            f.OpenBuffer(good[:cut])
        except N.NativeError:
            continue
        try:
            assert f.ReadEvent(1) == -1
        except N.NativeError:
            pass
    with pytest.raises(N.NativeError):
        ACorsikaIACTFile().OpenBuffer(os.urandom(256))
    # a bunch count that overruns its block
    bad = _long(0, [(1, 2, 0.1, 0.1, 0, 1e5, 1, 400)])
    bad = (0, bad[1][:8] + struct.pack("<i", 1000) + bad[1][12:])
    f = ACorsikaIACTFile()
    f.OpenBuffer(_stream([bad]))
    with pytest.raises(N.NativeError):
        f.ReadEvent(1)


def test_fixture_is_gzip_of_the_stream():
    raw = gzip.decompress(open(FIXTURE, "rb").read())
    f = ACorsikaIACTFile()
    f.OpenBuffer(raw)
    assert f.ReadEvent(1) == 1


# ---- GPU: bunch expansion and a traced event --------------------------------
@pytest.mark.gpu
def test_bunch_expansion_matches_oracle(event):
    z = 3000.0  # 30 m above the observation level, as tutorials/CORSIKA.C
    rays = event.GetDeviceRays(0, 0, z, 1.0, seed=17)
    got = {k: v.cpu().numpy() for k, v in rays.items()}
    b = event.GetBunches(0, 0)
    h = event.GetEventHeader()
    ref = oracle_ref.bunches_to_rays(b, z, event.GetTelescopeZ(0), 1.0, h.GetMinWavelength(), h.GetMaxWavelength(),
                                     17)
    n = int(np.sum(np.ceil(b["photons"][b["photons"] > 0])))
    assert len(got["x"]) == len(ref["x"]) == n
    for k in ("x", "y", "z", "t", "dx", "dy", "dz", "lam"):
        np.testing.assert_allclose(got[k], ref[k], rtol=1e-12, atol=1e-20, err_msg=k)
    lo, hi = h.GetMinWavelength() * 1e-7, h.GetMaxWavelength() * 1e-7
    assert (got["lam"] >= lo * (1 - 1e-12)).all() and (got["lam"] <= hi * (1 + 1e-12)).all()


@pytest.mark.gpu
def test_corsika_event_traced_like_oracle(event):
    import torch

    from robast_gb300 import device

    man, _ = configs.davies_cotton(n_rays=4, n_angles=1)
    rays = event.GetDeviceRays(0, 0, 3000.0, 1.0, seed=3)
    res, st = device.trace(man, rays, precision=N.PREC_MIXED)
    torch.cuda.synchronize()
    assert st == N.RBG_OK
    arr = event.GetRayArray(0, 0, 3000.0, 1.0, seed=3)
    ost, ref = oracle_ref.trace(man, arr, threads=8)
    assert ost == 0
    got = {k: v.cpu().numpy() for k, v in res.items()}
    same = (got["status"] == ref["status"]) & (got["npoints"] == ref["npoints"])
    assert same.mean() >= 0.999
    for k in ("x", "y", "z"):
        np.testing.assert_allclose(got[k][same], ref[k][same], rtol=1e-6, atol=1e-6)
