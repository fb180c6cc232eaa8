"""Writes zimg_gb300/csrc/blue_noise_table.inc from zimg's own build.

RANDOM dither adds entries of a fixed 64 x 64 blue-noise matrix
(src/zimg/depth/blue.h:10-13, used by dither.cpp:219-234). The matrix is data
with no generating rule, so results equal to zimg's need the same entries. This
script reads them out of the reference library built by `make -C oracle ref`
(oracle/_ref/libzimgref.so, export ref_blue_noise_table) and writes them as
1024 little-endian 32-bit words, four consecutive entries of a row per word,
the form the device kernel copies into shared memory.

    make -C oracle && python oracle/gen_blue_noise_table.py
"""
import ctypes
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "..", "zimg_gb300", "csrc", "blue_noise_table.inc")


def read_table() -> bytes:
    lib = ctypes.CDLL(os.path.join(HERE, "_ref", "libzimgref.so"))
    buf = (ctypes.c_uint8 * 4096)()
    lib.ref_blue_noise_table(buf)
    return bytes(buf)


def words(table: bytes) -> list:
    return [int.from_bytes(table[4 * k:4 * k + 4], "little") for k in range(1024)]


def render(table: bytes) -> str:
    w = words(table)
    lines = ["// zimg's 64 x 64 blue-noise matrix (src/zimg/depth/blue.h:10-13), written by",
             "// oracle/gen_blue_noise_table.py from zimg's own build: word k holds entries",
             "// 4k .. 4k+3 of the row-major matrix, entry 4k in the low byte."]
    for r in range(0, 1024, 8):
        lines.append("\t" + ", ".join(f"0x{v:08x}u" for v in w[r:r + 8]) + ",")
    return "\n".join(lines) + "\n"


def main() -> int:
    text = render(read_table())
    with open(OUT, "w") as f:
        f.write(text)
    print(f"wrote {os.path.normpath(OUT)}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
