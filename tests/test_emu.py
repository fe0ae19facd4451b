"""The integer-pipe IEEE double multiply that the bit-exact FP64 collision
uses for part of its products (porelb_gb300/csrc/plb_emu.h), built for the
CPU and checked bit for bit against the host's multiply: random operands of
wide range, ties to even, exact products, the collision's own kinds of
operands and signed zeros.  On the GPU the bit-exact tests check it inside
the collision."""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


def test_integer_multiply_equals_ieee(tmp_path):
    so = tmp_path / "emu_check.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                    "-o", str(so), os.path.join(HERE, "native", "emu_check.cpp")], check=True)
    lib = ctypes.CDLL(str(so))
    lib.emu_check.restype = ctypes.c_long
    lib.emu_check.argtypes = [ctypes.c_long, ctypes.c_ulonglong]
    assert lib.emu_check(1_000_000, 12345) == 0
