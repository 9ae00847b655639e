"""Minimal FITS primary-HDU image reader/writer (numpy only).

Imfit reads and writes FITS images through CFITSIO (reference
core/image_io.cpp:241-375).  This module covers what the model-image path
needs: a 2-D image HDU with BITPIX 8/16/32/-32/-64, BSCALE/BZERO, returned
as a float64 array indexed [row, column] with rows counted from the bottom of
the image (the order Imfit's pixel vectors use).  Names follow CFITSIO's
extended syntax as far as Imfit's tests use it: 'file.fits[N]' selects HDU
N (0 = primary), a plain name the primary HDU; an HDU without a 2-D image
is an error (core/image_io.cpp:160-171).  'file.fits[x1:x2,y1:y2]' selects
an image section, 'file.fits[N][x1:x2,y1:y2]' both.
"""
import re

import numpy as np

_BLOCK = 2880
_DT = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}


def _parse_header(raw, pos):
    cards = {}
    while True:
        block = raw[pos:pos + _BLOCK]
        if len(block) < _BLOCK:
            raise ValueError("truncated FITS header")
        pos += _BLOCK
        done = False
        for i in range(0, _BLOCK, 80):
            card = block[i:i + 80].decode("ascii", errors="replace")
            key = card[:8].strip()
            if key == "END":
                done = True
                break
            if card[8:10] == "= ":
                val = card[10:].split("/")[0].strip()
                if val.startswith("'"):
                    val = val.strip("'").strip()
                else:
                    try:
                        val = int(val)
                    except ValueError:
                        try:
                            val = float(val.replace("D", "E"))
                        except ValueError:
                            pass
                cards[key] = val
        if done:
            return cards, pos


def split_section(name):
    """'file.fits[x1:x2,y1:y2]' -> ('file.fits', (x1, x2, y1, y2)) with 1-based
    inclusive pixel ranges (x = column), as CFITSIO's image sections; a name
    without a section -> (name, None).  An HDU selector stays on the name."""
    m = re.fullmatch(r"(.*)\[\s*(\d+)\s*:\s*(\d+)\s*,\s*(\d+)\s*:\s*(\d+)\s*\]", name.strip())
    if not m:
        return name, None
    return m.group(1), tuple(int(m.group(i)) for i in range(2, 6))


def split_hdu(name):
    """'file.fits[N]' -> ('file.fits', N); a name without one -> (name, None)."""
    m = re.fullmatch(r"(.*)\[\s*(\d+)\s*\]", name.strip())
    if not m:
        return name, None
    return m.group(1), int(m.group(2))


def image_offset(name):
    """DetermineImageOffset (core/utilities.cpp:483-489): (x1 - 1, y1 - 1) of
    an image section, (0, 0) without one."""
    _, sec = split_section(name)
    return (0, 0) if sec is None else (sec[0] - 1, sec[2] - 1)


def read_image(path):
    """Return (float64 array [nrows, ncols], header dict) of the first 2-D image
    HDU; a trailing section [x1:x2,y1:y2] selects that part of the image."""
    path, sec = split_section(path)
    path, hdu = split_hdu(path)
    arr, hdr = _read_full(path, 0 if hdu is None else hdu)
    if sec is not None:
        x1, x2, y1, y2 = sec
        if not (1 <= x1 <= x2 <= arr.shape[1] and 1 <= y1 <= y2 <= arr.shape[0]):
            raise ValueError(f"image section {sec} outside the {arr.shape[1]} x {arr.shape[0]} image")
        arr = arr[y1 - 1:y2, x1 - 1:x2].copy()
    return arr, hdr


def _read_full(path, hdu=0):
    with open(path, "rb") as f:
        raw = f.read()
    pos, k = 0, 0
    while pos < len(raw):
        hdr, pos = _parse_header(raw, pos)
        naxis = int(hdr.get("NAXIS", 0))
        bitpix = int(hdr["BITPIX"])
        dims = [int(hdr.get(f"NAXIS{i + 1}", 0)) for i in range(naxis)]
        nbytes = abs(bitpix) // 8 * (int(np.prod(dims)) if naxis else 0)
        image = naxis == 2 and nbytes > 0 and hdr.get("XTENSION", "IMAGE") in ("IMAGE", None)
        if image and hdu == k:
            data = np.frombuffer(raw, dtype=_DT[bitpix], count=int(np.prod(dims)), offset=pos)
            arr = data.astype(np.float64).reshape(dims[1], dims[0])
            arr = arr * float(hdr.get("BSCALE", 1.0)) + float(hdr.get("BZERO", 0.0))
            return arr, hdr
        if hdu == k:
            break
        pos += ((nbytes + _BLOCK - 1) // _BLOCK) * _BLOCK
        k += 1
    raise ValueError(f"Unable to find valid 2D image in extension {hdu} (HDU {hdu + 1}) of {path}")


def write_image(path, arr, bitpix=-32):
    """Write a 2-D array as a primary-HDU FITS image (float32 by default)."""
    arr = np.asarray(arr)
    nrows, ncols = arr.shape
    cards = [("SIMPLE", "T"), ("BITPIX", str(bitpix)), ("NAXIS", "2"), ("NAXIS1", str(ncols)),
             ("NAXIS2", str(nrows))]
    hdr = "".join(f"{k:<8}= {v:>20}".ljust(80) for k, v in cards) + "END".ljust(80)
    hdr = hdr.ljust(((len(hdr) + _BLOCK - 1) // _BLOCK) * _BLOCK)
    body = np.ascontiguousarray(arr, dtype=_DT[bitpix]).tobytes()
    body += b"\0" * ((-len(body)) % _BLOCK)
    with open(path, "wb") as f:
        f.write(hdr.encode("ascii") + body)
