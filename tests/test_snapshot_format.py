"""The snapshot file format (ramgpu_save_state / ramgpu_load_state), checked
without a GPU: a file written here by an independent writer of the
documented layout is accepted by the library's context-free reader
ramgpu_snapshot_info, and damaged files are rejected with RAMGPU_ERR_IO."""
import struct

import numpy as np
import pytest

from ramgpu import abi

NR, NT, NE, NPA, NS, NM = 4, 5, 3, 6, 2, 3


def _fnv_words(payload: bytes) -> int:
    h = 1469598103934665603
    for (w,) in struct.iter_unpack("<Q", payload):
        h = ((h ^ w) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def _payload(rng):
    parts = []
    for m in range(NM):
        parts.append(struct.pack("<4i", 0b11, 1, 1, 0))
        parts.append(struct.pack("<d", 2.0 + m))
        parts.append(rng.random((NR + 1) * NT).tobytes())
    for _ in range(NM * NS):
        parts.append(rng.random(NR * NT * NE * NPA + NT * NE * NPA + 2 * NR * NT).tobytes())
    return b"".join(parts)


def _write(path, payload, time=1234.5, magic=b"RAMGPUS1", version=1, checksum=None):
    hdr = magic + struct.pack("<2I6i2Id2Q", version, 128, NR, NT, NE, NPA, NS, NM, 5, 0, time, len(payload),
                              _fnv_words(payload) if checksum is None else checksum)
    hdr += b"\0" * (128 - len(hdr))
    path.write_bytes(hdr + payload)


def test_reader_accepts_the_documented_layout(tmp_path):
    p = tmp_path / "ok.snap"
    _write(p, _payload(np.random.Generator(np.random.PCG64(1))))
    info = abi.snapshot_info(p)
    assert (info["nr"], info["nt"], info["ne"], info["npa"], info["ns"], info["n_members"]) == (NR, NT, NE, NPA, NS, NM)
    assert info["flags"] == 5 and info["time"] == 1234.5


@pytest.mark.parametrize("damage", ["flip", "truncate", "magic", "version", "size"])
def test_reader_rejects_damaged_files(tmp_path, damage):
    rng = np.random.Generator(np.random.PCG64(2))
    payload = _payload(rng)
    p = tmp_path / "bad.snap"
    if damage == "magic":
        _write(p, payload, magic=b"RAMGPUS0")
    elif damage == "version":
        _write(p, payload, version=2)
    elif damage == "size":
        _write(p, payload[:-8], checksum=_fnv_words(payload[:-8]))  # consistent checksum, wrong payload size
    else:
        _write(p, payload)
        raw = bytearray(p.read_bytes())
        if damage == "flip":
            raw[128 + len(payload) // 2] ^= 0x10
        else:
            raw = raw[:-16]
        p.write_bytes(bytes(raw))
    with pytest.raises(abi.RamGpuError) as e:
        abi.snapshot_info(p)
    assert e.value.code == -6


def test_reader_missing_file(tmp_path):
    with pytest.raises(abi.RamGpuError) as e:
        abi.snapshot_info(tmp_path / "none.snap")
    assert e.value.code == -6
