"""Generate ``basis_sets.json`` from the reference's basis-set data files.

The reference ships every basis twice (``data/basis/*.basis`` and
``data/basis_text/*.txt``):

* the cereal-serialised blobs that ``fetchBasis``
  (Science/QuantumChemistry/BasisSet/FetchBasis.hs:63-73) decodes at run time.
  They were written by ``parseBasis`` whose ``triple`` helper
  (Science/QuantumChemistry/ParsecTools/ParserBasis.hs:116-118) stores the
  constant 1.0 in place of the exponent of every SP primitive.  This variant is
  recorded as ``"shipped"``: it is what the reference's own SCF runs on.
* the EMSL text the blobs were made from, parsed here with the exponent kept.
  This variant is recorded as ``"text"`` (physically meaningful numbers).

Each shell is written as ``{"kind": "S"|"SP"|"P"|"D", "exps": [...],
"coefs": [[...], ...]}`` with raw (unnormalised) contraction coefficients; the
primitive normalisation of ``normCoeff`` (NormalizeBasis.hs:52-59) is applied
by the host code that builds CGFs (``gbhf.basis``).

Run once in a container that holds the reference checkout::

    python make_basis_data.py /path/to/reference/data > basis_sets.json
"""
import json
import struct
import sys
from pathlib import Path

ELEMENTS = ("H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne")
BASES = {"sto-3g": "sto-3g", "3-21g": "3-21g", "6-31g": "6-31g", "6-31g*": "6-31gs", "6-31g**": "6-31gss",
         "6-31++g*": "6-31mmgs"}
TAGS = {0: "S", 1: "SP", 2: "P", 3: "D"}


class _Reader:
    """Big-endian reader for the cereal encoding of ``[Element]``."""

    def __init__(self, data):
        self.data, self.pos = data, 0

    def u64(self):
        (v,) = struct.unpack_from(">Q", self.data, self.pos)
        self.pos += 8
        return v

    def u8(self):
        v = self.data[self.pos]
        self.pos += 1
        return v

    def f64(self):
        (v,) = struct.unpack_from(">d", self.data, self.pos)
        self.pos += 8
        return v

    def bytes_(self):
        n = self.u64()
        v = self.data[self.pos:self.pos + n]
        self.pos += n
        return v


def decode_blob(data):
    """Decode a ``.basis`` blob: list of ``Atom label [GaussShape]``."""
    r = _Reader(data)
    out = {}
    for _ in range(r.u64()):
        label = r.bytes_().decode()
        shells = []
        for _ in range(r.u64()):
            kind = TAGS[r.u8()]
            n = r.u64()
            if kind == "SP":
                prims = [(r.f64(), r.f64(), r.f64()) for _ in range(n)]  # (c_s, c_p, e)
                shells.append({"kind": "SP", "exps": [p[2] for p in prims],
                               "coefs": [[p[0] for p in prims], [p[1] for p in prims]]})
            else:
                prims = [(r.f64(), r.f64()) for _ in range(n)]  # (c, e)
                shells.append({"kind": kind, "exps": [p[1] for p in prims],
                               "coefs": [[p[0] for p in prims]]})
        out[label] = shells
    assert r.pos == len(data)
    return out


def parse_text(text):
    """Parse the EMSL NWChem-format text, keeping the SP exponents."""
    out = {}
    lines = text.splitlines()
    i = 0
    while i < len(lines) and not lines[i].startswith('BASIS "ao basis"'):
        i += 1
    i += 1
    cur = None
    for line in lines[i:]:
        toks = line.split()
        if not toks or line.startswith("#") or toks[0] == "END":
            continue
        if toks[0].isalpha():
            label, kind = toks[0], toks[1]
            cur = {"kind": "S" if kind == "S" else kind, "rows": []}
            out.setdefault(label, []).append(cur)
            continue
        cur["rows"].append([float(t.replace("D", "E")) for t in toks])
    res = {}
    for label, shells in out.items():
        res[label] = []
        for sh in shells:
            rows = sh["rows"]
            ncol = len(rows[0]) - 1
            res[label].append({"kind": sh["kind"], "exps": [r[0] for r in rows],
                               "coefs": [[r[1 + c] for r in rows] for c in range(ncol)]})
    return res


def main(root):
    root = Path(root)
    result = {"source": "EMSL basis data as shipped in the reference (data/basis, data/basis_text)",
              "sets": {}}
    for name, fname in BASES.items():
        shipped = decode_blob((root / "basis" / f"{fname}.basis").read_bytes())
        text = parse_text((root / "basis_text" / f"{fname}.txt").read_text())
        result["sets"][name] = {
            "shipped": {e: shipped[e] for e in ELEMENTS if e in shipped},
            "text": {e: text[e] for e in ELEMENTS if e in text},
        }
    json.dump(result, sys.stdout, indent=1)
    sys.stdout.write("\n")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: python make_basis_data.py <reference checkout>/data > basis_sets.json")
    main(sys.argv[1])
