"""ILDG / SciDAC gauge files restated in numpy (TEST INFRASTRUCTURE ONLY: the checker for
the library's reader and writer; only tests/ use it).

Follows Grid/parallelIO/IldgIO.h:611-950 (record sequence, required records, checks) and
the SciDAC checksum of Grid/parallelIO/BinaryIO.h:139-192.  The LIME container is the
c-lime library's published format (Grid links it; it is not in Grid's sources): per
record a 144-byte big-endian header (magic 0x456789ab, version 1, flags with 0x8000 =
message begin and 0x4000 = message end, 8-byte data length, 128-byte type), then the data
padded to 8 bytes.  CRC-32 here is Python's zlib.crc32, an implementation independent of
the library's device CRC.
"""
from __future__ import annotations

import re
import struct
import zlib

import numpy as np

from oracle import nersc

MAGIC = 0x456789AB


def lime_records(path):
    """[(type, mb, me, data offset, data length)] of every record in the file."""
    out = []
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos + 144 <= len(data):
        magic, version, flags, n = struct.unpack(">IHHQ", data[pos:pos + 16])
        assert magic == MAGIC, f"no LIME record at {pos}"
        rtype = data[pos + 16:pos + 144].split(b"\0", 1)[0].decode()
        out.append((rtype, bool(flags & 0x8000), bool(flags & 0x4000), pos + 144, n))
        pos += 144 + (n + 7) // 8 * 8
    return out


def _record(rtype, payload: bytes, mb=False, me=False):
    hdr = struct.pack(">IHHQ", MAGIC, 1, (0x8000 if mb else 0) | (0x4000 if me else 0), len(payload))
    hdr += rtype.encode().ljust(128, b"\0")
    return hdr + payload + b"\0" * ((8 - len(payload) % 8) % 8)


def scidac_checksum(site_bytes: np.ndarray):
    """suma, sumb of a (vol, nbytes) uint8 array of the sites as stored."""
    a = b = 0
    for s in range(site_bytes.shape[0]):
        crc = zlib.crc32(site_bytes[s].tobytes()) & 0xFFFFFFFF
        r29, r31 = s % 29, s % 31
        a ^= ((crc << r29) | (crc >> (32 - r29))) & 0xFFFFFFFF if r29 else crc
        b ^= ((crc << r31) | (crc >> (32 - r31))) & 0xFFFFFFFF if r31 else crc
    return a, b


def _site_bytes(U, dims, precision):
    vol = int(np.prod(dims))
    dt = ">c16" if precision == 64 else ">c8"
    return np.ascontiguousarray(np.asarray(U).reshape(vol, 36).astype(dt)).view(np.uint8).reshape(vol, -1)


def write(path, U, dims, precision=64, lfn="", with_checksum=True, plaquette=None):
    """The record sequence of IldgWriter::writeConfiguration without Grid's private records."""
    dims = list(dims)
    sb = _site_bytes(U, dims, precision)
    suma, sumb = scidac_checksum(sb)
    if plaquette is None:
        plaquette = nersc.plaquette_and_trace(np.asarray(U).reshape(-1, 4, 3, 3), dims)
    plaq, trace = float(plaquette[0]), float(plaquette[1])
    usqcd = (f'<?xml version="1.0"?>\n<usqcdInfo><version>1</version><plaq>{plaq!r}</plaq>'
             f"<linktr>{trace!r}</linktr><info>oracle</info></usqcdInfo>").encode()
    recs = [
        _record("scidac-private-file-xml",
                (f'<?xml version="1.0"?>\n<scidacFile><version>1.1</version><spacetime>4</spacetime>'
                 f"<dims>{' '.join(map(str, dims))} </dims><volfmt>0</volfmt></scidacFile>").encode(), mb=True),
        _record("scidac-file-xml", usqcd, me=True),
        _record("scidac-private-record-xml", b'<?xml version="1.0"?>\n<scidacRecord><version>1.1</version>'
                b"<recordtype>0</recordtype></scidacRecord>", mb=True),
        _record("scidac-record-xml", usqcd),
        _record("ildg-format", (f'<?xml version="1.0" encoding="UTF-8"?>\n<ildgFormat xmlns="http://www.lqcd.org/ildg">'
                                f"<version>1.0</version><field>su3gauge</field><precision>{precision}</precision>"
                                f"<lx>{dims[0]}</lx><ly>{dims[1]}</ly><lz>{dims[2]}</lz><lt>{dims[3]}</lt>"
                                f"</ildgFormat>").encode()),
        _record("ildg-data-lfn", lfn.encode()),
        _record("ildg-binary-data", sb.tobytes()),
    ]
    if with_checksum:
        recs.append(_record("scidac-checksum", (f'<?xml version="1.0"?>\n<scidacChecksum><version>1</version>'
                                                f"<suma>{suma:x}</suma><sumb>{sumb:x}</sumb></scidacChecksum>").encode(),
                            me=True))
    with open(path, "wb") as f:
        f.write(b"".join(recs))
    return suma, sumb


def _tag(xml, tag):
    m = re.search(rf"<{tag}(\s[^>]*)?>(.*?)</{tag}>", xml, re.S)
    return m.group(2).strip() if m else None


def read(path):
    """(U canonical complex128 [site][mu][3][3] flattened, meta dict); meta holds the file's
    and the recomputed checksums."""
    meta = {}
    with open(path, "rb") as f:
        data = f.read()
    raw = None
    for rtype, _, _, off, n in lime_records(path):
        body = data[off:off + n]
        if rtype.startswith("ildg-binary-data"):
            raw = body
            continue
        text = body.split(b"\0", 1)[0].decode()
        if rtype.startswith("ildg-format"):
            meta["precision"] = int(_tag(text, "precision"))
            meta["dims"] = [int(_tag(text, t)) for t in ("lx", "ly", "lz", "lt")]
            meta["field"] = _tag(text, "field")
        elif rtype.startswith("ildg-data-lfn"):
            meta["lfn"] = text
        elif rtype.startswith("scidac-checksum"):
            meta["suma"], meta["sumb"] = int(_tag(text, "suma"), 16), int(_tag(text, "sumb"), 16)
        elif rtype.startswith("scidac-record-xml") and "usqcdInfo" in text:
            meta["plaquette"], meta["link_trace"] = float(_tag(text, "plaq")), float(_tag(text, "linktr"))
    vol = int(np.prod(meta["dims"]))
    dt = ">c16" if meta["precision"] == 64 else ">c8"
    arr = np.frombuffer(raw, dtype=dt)
    meta["suma_computed"], meta["sumb_computed"] = scidac_checksum(np.frombuffer(raw, dtype=np.uint8).reshape(vol, -1))
    return arr.astype(np.complex128), meta
