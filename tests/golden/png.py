"""Minimal PNG decoder (8-bit gray/RGB/RGBA, non-interlaced) with zlib and
numpy, used to read the reference's golden images. Test infrastructure."""
import struct
import zlib

import numpy as np


def _paeth_row(line, prev, bpp):
  out = np.zeros_like(line)
  for x in range(line.shape[0]):
    a = int(out[x - bpp]) if x >= bpp else 0
    b = int(prev[x])
    c = int(prev[x - bpp]) if x >= bpp else 0
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
    out[x] = (int(line[x]) + pr) & 255
  return out


def read_png(path):
  return decode_png(open(path, "rb").read(), path)


def decode_png(data, name="<bytes>"):
  """Decodes the bytes of a PNG file (bytes or a uint8 array)."""
  data = bytes(np.asarray(bytearray(data) if isinstance(data, bytes) else data, np.uint8))
  if data[:8] != b"\x89PNG\r\n\x1a\n":
    raise ValueError("not a PNG: %s" % name)
  pos, idat = 8, b""
  while pos < len(data):
    (n,) = struct.unpack(">I", data[pos:pos + 4])
    kind = data[pos + 4:pos + 8]
    body = data[pos + 8:pos + 8 + n]
    pos += 12 + n
    if kind == b"IHDR":
      w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
    elif kind == b"IDAT":
      idat += body
  if depth != 8 or interlace != 0:
    raise ValueError("only 8-bit non-interlaced PNGs are supported")
  ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
  raw = np.frombuffer(zlib.decompress(idat), np.uint8)
  stride = w * ch
  out = np.zeros((h, stride), np.uint8)
  prev = np.zeros(stride, np.uint8)
  p = 0
  for y in range(h):
    f = raw[p]
    line = raw[p + 1:p + 1 + stride].astype(np.int64)
    p += 1 + stride
    if f == 0:
      cur = line
    elif f == 1:
      cur = line.reshape(w, ch).cumsum(0).reshape(-1)
    elif f == 2:
      cur = line + prev
    elif f == 3:
      cur = np.zeros(stride, np.int64)
      for x in range(stride):
        a = cur[x - ch] if x >= ch else 0
        cur[x] = (line[x] + ((int(a) + int(prev[x])) >> 1)) & 255
    else:
      cur = _paeth_row(line.astype(np.uint8), prev, ch)
    cur = (np.asarray(cur) & 255).astype(np.uint8)
    out[y] = cur
    prev = cur
  return out.reshape(h, w, ch)
