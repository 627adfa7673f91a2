"""Generate tests/golden/golden.json from an openLOWDIN source tree.

Run once in a container that has the reference tree:

    python tests/golden/make_golden.py [REFERENCE_ROOT]

REFERENCE_ROOT defaults to $LOWDIN_REFERENCE, else /root/reference.

It extracts, as data:
  * the basis-set entries the golden tests use from ``lib/basis`` (6-311G for
    H and O electrons, NAKAI-5-SPD for quantum protons),
  * the geometries of the golden inputs ``test/H2O.BOA.DIRECT.lowdin``,
    ``test/H2O.APMO.MP2.lowdin`` (Angstrom, converted with AMSTRONG =
    0.52917724924 bohr from ``src/core/Units.f90:37``),
  * the golden values asserted by the checkers ``test/H2O.BOA.DIRECT.py``,
    ``test/H2O.BOA.MP2.DIRECT.py``, ``test/H2O.APMO.MP2.py``,
    ``test/H2O.APMO.UHF.DIRECT.py``, ``test/H2O.APMO.UMP2.DIRECT.py`` (the
    last two use the geometry of ``test/H2O.APMO.MP2.lowdin``).
The GPU machine has no reference tree, so the tests read only the JSON written here.
"""
import json
import os
import re
import sys

ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LOWDIN_REFERENCE", "/root/reference")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
BOHR = 0.52917724924  # src/core/Units.f90:37


def read_basis(fname, element, symbol):
    """Parse one entry 'O-<ELEMENT> <SYMBOL> (<NAME>) BASIS TYPE: n' of a lowdin
    basis file: '#' line, shell count, then per shell 'id l nprim' and nprim
    'exponent coefficient' rows (src/core/BasisSet.f90:180-250)."""
    lines = open(os.path.join(ROOT, "lib", "basis", fname)).read().splitlines()
    head = re.compile(r"^O-%s\s+%s\s+\(" % (re.escape(element), re.escape(symbol)))
    for i, ln in enumerate(lines):
        if head.match(ln.strip()):
            j = i + 1
            while lines[j].strip().startswith("#"):
                j += 1
            nsh = int(lines[j].split()[0]); j += 1
            shells = []
            for _ in range(nsh):
                _, l, npr = (int(x) for x in lines[j].split()[:3]); j += 1
                ex, co = [], []
                for _ in range(npr):
                    a, c = lines[j].split()[:2]; j += 1
                    ex.append(float(a.replace("D", "E"))); co.append(float(c.replace("D", "E")))
                shells.append({"l": l, "exponents": ex, "coefficients": co})
            return shells
    raise KeyError(f"{element} {symbol} not in {fname}")


def read_geometry(name):
    rows = []
    txt = open(os.path.join(ROOT, "test", name)).read()
    block = txt.split("GEOMETRY")[1]
    for ln in block.splitlines()[1:]:
        ln = ln.strip()
        if not ln or ln.startswith("END"):
            break
        parts = ln.split()
        rec = {"particle": parts[0], "basis": parts[1],
               "position_bohr": [float(x) / BOHR for x in parts[2:5]]}
        m = re.search(r"m\s*=\s*([0-9.Ee+-]+)", ln)
        if m:
            rec["mass"] = float(m.group(1))
        rows.append(rec)
    return rows


def read_checker(name):
    txt = open(os.path.join(ROOT, "test", name)).read()
    vals = {}
    m = re.search(r"refTotalEnergy\s*=\s*([-0-9.Ee+]+)", txt)
    if m:
        vals["HF energy"] = [float(m.group(1)), 1e-8]
    m = re.search(r"refMP2Energy\s*=\s*([-0-9.Ee+]+)", txt)
    if m:
        vals["MP2 energy"] = [float(m.group(1)), 1e-5]
    for key, val, tol in re.findall(r'"([^"]+)"\s*:\s*\[\s*([-0-9.Ee+]+)\s*,\s*([-0-9.Ee+]+)\s*\]', txt):
        vals[key] = [float(val), float(tol)]
    return vals


def main():
    data = {
        "source": "generated by tests/golden/make_golden.py from the openLOWDIN tree",
        "basis": {
            "6-311G:H": read_basis("6-311G", "HYDROGEN", "H"),
            "6-311G:O": read_basis("6-311G", "OXYGEN", "O"),
            "NAKAI-5-SPD:H_1": read_basis("NAKAI-5-SPD", "HYDROGEN_1", "H_1"),
        },
        "geometry": {
            "H2O.BOA.DIRECT": read_geometry("H2O.BOA.DIRECT.lowdin"),
            "H2O.APMO.MP2": read_geometry("H2O.APMO.MP2.lowdin"),
        },
        "values": {
            "H2O.BOA.DIRECT": read_checker("H2O.BOA.DIRECT.py"),
            "H2O.BOA.MP2.DIRECT": read_checker("H2O.BOA.MP2.DIRECT.py"),
            "H2O.APMO.MP2": read_checker("H2O.APMO.MP2.py"),
            "H2O.APMO.UHF.DIRECT": read_checker("H2O.APMO.UHF.DIRECT.py"),
            "H2O.APMO.UMP2.DIRECT": read_checker("H2O.APMO.UMP2.DIRECT.py"),
        },
    }
    with open(OUT, "w") as f:
        json.dump(data, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
