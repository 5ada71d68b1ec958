"""BGZF writer for the tests: gzip members of at most 64 KiB, each with the
'BC' extra subfield holding the member's size, then the empty end-of-file
member (the layout bgzip writes).  The result is also ordinary multi-member
gzip, so zlib reads it too."""
import struct
import zlib


def member(data: bytes, level: int) -> bytes:
    co = zlib.compressobj(level, zlib.DEFLATED, -15)
    cdata = co.compress(data) + co.flush()
    bsize = 18 + len(cdata) + 8 - 1
    head = struct.pack("<BBBBIBBHBBHH", 31, 139, 8, 4, 0, 0, 255, 6, ord("B"), ord("C"), 2, bsize)
    return head + cdata + struct.pack("<II", zlib.crc32(data) & 0xFFFFFFFF, len(data))


def bgzf(data: bytes, level: int = 6, block: int = 65280, eof: bool = True) -> bytes:
    out = [member(data[i:i + block], level) for i in range(0, len(data), block)]
    if eof:
        out.append(member(b"", level))
    return b"".join(out)
