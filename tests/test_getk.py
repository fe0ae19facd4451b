"""getK's analytic BCC permeability, restated in porelb_gb300.getk, against
the reference's getK.c.  getK.c does not compile as shipped (two statements
lack their semicolons, getK.c:53-54); when the reference tree is present this
test compiles a temporary copy with exactly those two characters added."""
import os
import re
import subprocess

import pytest

from porelb_gb300 import getk



def _ref_dir():
    """The reference tree: $REF_DIR, else the one oracle/Makefile built
    oracle/_ref from (recorded in oracle/_ref/REF_DIR); '' when neither."""
    d = os.environ.get("REF_DIR", "")
    if not d:
        rec = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                           "oracle", "_ref", "REF_DIR")
        if os.path.exists(rec):
            with open(rec) as fh:
                d = fh.read().strip()
    return d


REF = os.path.join(_ref_dir(), "getK.c") if _ref_dir() else ""


def test_series_and_porosity():
    k1a, k2a, a, eps = getk.bcc_k(0.5, 63.0)
    k1b, _, _, _ = getk.bcc_k(0.8, 63.0)
    assert 0 < eps < 1 and k1b < k1a  # larger spheres, lower permeability
    assert abs(a - 3 ** 0.5 * 63.0 * 0.5 / 4) < 1e-12
    assert len(getk.QS_BCC) == 31 and getk.QS_BCC[0] == 1.0


@pytest.mark.skipif(not REF or not os.path.exists(REF), reason="reference tree not present")
@pytest.mark.parametrize("chi,nx", [("0.3", "64"), ("0.6", "128"), ("0.95", "33")])
def test_getk_matches_reference_program(tmp_path, chi, nx):
    src = open(REF).read()
    fixed = src.replace('printf("Usage: ./testpre Chi nx\\n")\n',
                        'printf("Usage: ./testpre Chi nx\\n");\n')
    fixed = fixed.replace('printf("0<Chi<1 controls the size of the sphere, and nx is the resolution\\n")\n',
                          'printf("0<Chi<1 controls the size of the sphere, and nx is the resolution\\n");\n')
    assert fixed.count(";") == src.count(";") + 2
    c = tmp_path / "getK.c"
    c.write_text(fixed)
    exe = tmp_path / "getK"
    subprocess.run(["gcc", "-O2", "-o", str(exe), str(c), "-lm"], check=True)
    out = subprocess.run([str(exe), chi, nx], capture_output=True, text=True,
                         check=True).stdout
    k1 = float(re.search(r"K1=(\S+)", out).group(1))
    k2 = float(re.search(r"K2=(\S+)", out).group(1))
    m1, m2, _, _ = getk.getk(float(chi), int(nx))
    assert abs(m1 - k1) <= 1e-6 * abs(k1)  # printed with %e (7 digits)
    assert abs(m2 - k2) <= 1e-6 * abs(k2)
