"""The Python mirror of the flat layout matches include/posidonius_gb300.h."""
import os
import re

from posidonius_gb300 import layout as L

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "posidonius_gb300.h")


def _enums():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for body in re.findall(r"enum\s+\w+\s*\{(.*?)\};", text, flags=re.S):
        value = -1
        for item in body.split(","):
            item = item.strip()
            if not item:
                continue
            if "=" in item:
                name, expr = [x.strip() for x in item.split("=", 1)]
                value = eval(expr.replace("<<", "<<"), {}, out)
            else:
                name = item
                value += 1
            out[name] = value
    return out


def test_every_header_constant_is_mirrored():
    enums = _enums()
    assert len(enums) > 80
    for name, value in enums.items():
        assert name.startswith("POSI_")
        short = name[len("POSI_"):]
        if short.startswith("MODE_") or short.startswith("MAP_"):
            pass
        assert hasattr(L, short), short
        assert getattr(L, short) == value, (short, getattr(L, short), value)


def test_max_bodies():
    text = open(HEADER).read()
    m = re.search(r"#define\s+POSI_MAX_BODIES\s+(\d+)", text)
    assert int(m.group(1)) == L.MAX_BODIES


def test_ln2_split_constants():
    """The double-double ln 2 of the kernels' exp (kLN2_HI + kLN2_LO) equals
    ln 2 to about 2^-106."""
    import decimal
    import os
    import re
    src = open(os.path.join(os.path.dirname(__file__), "..", "posidonius_gb300", "csrc", "whfast_device.cuh")).read()
    hi = float.fromhex(re.search(r"kLN2_HI = (0x[0-9a-fp.+-]+);", src).group(1))
    lo = float.fromhex(re.search(r"kLN2_LO = (0x[0-9a-fp.+-]+);", src).group(1))
    decimal.getcontext().prec = 60
    ln2 = decimal.Decimal(2).ln()
    err = abs(decimal.Decimal(hi) + decimal.Decimal(lo) - ln2)
    assert hi == float(ln2)
    assert err < decimal.Decimal(2) ** -106
