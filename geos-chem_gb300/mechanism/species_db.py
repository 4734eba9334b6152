"""Per-species physical constants of a KPP mechanism from GEOS-Chem's species
database (run/shared/species_database.yml): MW_g, Henry_K0 and Henry_CR,
which Do_FullChem copies into the KPP arrays MW, SR_MW, HENRY_K0 and
HENRY_CR for the heterogeneous rate laws (GeosCore/fullchem_mod.F90:2911-2920;
species absent from the database keep 0).

    python -m gcchem.mechanism.species_db <reference root> [mech]

writes ``mechanism/<mech>_species.json`` ({"species", "mw", "henry_k0",
"henry_cr"} in KPP species order).  The reader handles the subset of YAML
the database uses: top-level species blocks of ``key: value`` lines, anchors
(``NAME: &anchor``) and merges (``<< : *anchor``).
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FIELDS = ("MW_g", "Henry_K0", "Henry_CR")


def read_database(path):
    blocks, anchors, merges = {}, {}, {}
    cur = None
    with open(path) as fh:
        for line in fh:
            line = line.split(" #")[0].rstrip() if not line.startswith("#") else ""
            if not line.strip():
                continue
            m = re.match(r"^'?([A-Za-z0-9_\-]+)'?:\s*(&(\S+))?\s*$", line)
            if m:
                cur = m.group(1)
                blocks[cur] = {}
                if m.group(3):
                    anchors[m.group(3)] = cur
                continue
            m = re.match(r"^\s+<<\s*:\s*\*(\S+)\s*$", line)
            if m and cur:
                merges.setdefault(cur, []).append(m.group(1))
                continue
            m = re.match(r"^\s+([A-Za-z0-9_]+):\s*(.*)$", line)
            if m and cur:
                blocks[cur][m.group(1)] = m.group(2).strip()

    def resolved(name, depth=0):
        out = {}
        for a in merges.get(name, []):
            if depth < 8 and a in anchors:
                out.update(resolved(anchors[a], depth + 1))
        out.update(blocks[name])
        return out

    return {name: resolved(name) for name in blocks}


def constants(db, species):
    out = {"species": list(species)}
    for f, key in zip(FIELDS, ("mw", "henry_k0", "henry_cr")):
        vals = []
        for s in species:
            v = db.get(s, {}).get(f)
            vals.append(float(v) if v not in (None, "") else 0.0)
        out[key] = vals
    return out


def write(root, mech="fullchem"):
    with open(os.path.join(HERE, mech + ".json")) as fh:
        species = json.load(fh)["species"]
    db = read_database(os.path.join(root, "run", "shared", "species_database.yml"))
    out = constants(db, species)
    path = os.path.join(HERE, mech + "_species.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=0)
    return path


def load(mech="fullchem"):
    with open(os.path.join(HERE, mech + "_species.json")) as fh:
        return json.load(fh)


if __name__ == "__main__":
    print(write(sys.argv[1], sys.argv[2] if len(sys.argv) > 2 else "fullchem"))
