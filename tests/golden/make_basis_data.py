"""Convert the basis sets the workloads need (STO-3G, 6-31G, 6-31G* for H, C, N, O) from
the reference's example GAMESS-UK files into gaussium_gb300/data/basis_sets.json.

Basis-set exponents and contraction coefficients are published data (Hehre, Stewart &
Pople 1969; Hehre, Ditchfield & Pople 1972; Hariharan & Pople 1973); 6-31G is 6-31G*
without its d shells.  Run once, with GAUSSIUM_REFERENCE set to the reference source tree:
    GAUSSIUM_REFERENCE=<tree> python make_basis_data.py
"""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "..", "..", "gaussium_gb300", "data", "basis_sets.json")
ELEMENTS = {"HYDROGEN": "H", "CARBON": "C", "NITROGEN": "N", "OXYGEN": "O", "HELIUM": "He"}


def parse(path):
    blocks, cur = {}, None
    for raw in open(path).read().splitlines():
        line = raw.strip()
        if not line:
            continue
        if line.startswith("#"):
            w = line[1:].strip().split()
            cur = w[0].upper() if w and w[0].upper() in ELEMENTS else None
            if cur:
                blocks[cur] = []
            continue
        if cur is None:
            continue
        p = line.split()
        if p[0] in ("S", "L", "P", "D"):
            blocks[cur].append({"type": p[0], "rows": []})
        else:
            blocks[cur][-1]["rows"].append([float(x) for x in p])
    return {ELEMENTS[k]: v for k, v in blocks.items()}


def main():
    root = os.environ.get("GAUSSIUM_REFERENCE")
    if not root:
        raise SystemExit("set GAUSSIUM_REFERENCE to the reference source tree")
    REF = os.path.join(root, "examples", "basissets")
    sto = parse(os.path.join(REF, "STO-3G.gbs"))
    p631s = parse(os.path.join(REF, "6-31GP.gbs"))
    p631 = {el: [s for s in shells if s["type"] != "D"] for el, shells in p631s.items()}
    data = {"STO-3G": sto, "6-31G*": p631s, "6-31G": p631}
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    with open(OUT, "w") as f:
        json.dump(data, f, indent=0)


if __name__ == "__main__":
    main()
