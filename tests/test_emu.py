"""The integer-pipe IEEE double multiply that the bit-exact FP64 collision
uses for part of its products (porelb_gb300/csrc/plb_emu.h), built for the
CPU and checked bit for bit against the host's multiply: random operands of
wide range, ties to even, exact products, the collision's own kinds of
operands and signed zeros; the unchecked in-domain multiply and the node
range check the collision uses to call it.  On the GPU the bit-exact tests
check it inside the collision."""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


import pytest


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    so = tmp_path_factory.mktemp("emu") / "emu_check.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                    "-o", str(so), os.path.join(HERE, "native", "emu_check.cpp")], check=True)
    lib = ctypes.CDLL(str(so))
    lib.emu_check.restype = ctypes.c_long
    lib.emu_check.argtypes = [ctypes.c_long, ctypes.c_ulonglong]
    lib.fast_check.restype = ctypes.c_long
    lib.fast_check.argtypes = [ctypes.c_long, ctypes.c_ulonglong]
    lib.node_range_check.restype = ctypes.c_long
    lib.node_range_check.argtypes = [ctypes.c_long, ctypes.c_ulonglong,
                                     ctypes.POINTER(ctypes.c_long)]
    return lib


def test_integer_multiply_equals_ieee(emu):
    assert emu.emu_check(1_000_000, 12345) == 0


def test_unchecked_multiply_in_domain_and_range_test(emu):
    assert emu.fast_check(1_000_000, 777) == 0


def test_node_range_keeps_every_product_in_domain(emu):
    """The collision's node check (its values, density and run constants
    zero or in [2^-64, 2^64)) is what lets it multiply without checks: over
    nodes that pass it, including values at the ends of the range and
    densities cancelled down to 2^-64, no integer-path product leaves the
    multiply's domain."""
    checked = ctypes.c_long(0)
    assert emu.node_range_check(400_000, 99, ctypes.byref(checked)) == 0
    assert checked.value > 100_000
