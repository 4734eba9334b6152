"""Extract the record layout of GEOS-Chem's KPP-Standalone state files from
the reference writer (GeosCore/kppsa_interface_mod.F90, KppSa_Write_Samples)
into tests/golden/kppsa_layout.json: the labelled header lines with their
Fortran edit descriptors, the option rows, and the FORMATs of the CSV rows.
tests/test_kppsa.py checks gcchem.kppsa.write_state against it.

    python tests/golden/make_kppsa_layout.py [REFERENCE_ROOT]

REFERENCE_ROOT defaults to $GC_REFERENCE_ROOT, else /root/reference.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def extract(src):
    text = open(src).read()
    body = text[text.index("SUBROUTINE KppSa_Write_Samples"):text.index("END SUBROUTINE KppSa_Write_Samples")]
    body = re.sub(r"&\s*\n\s*", " ", body)  # join continuation lines
    body = body[body.rindex("WRITE", 0, body.index("Meteorological and general grid cell metadata")):]
    lines = []
    for m in re.finditer(r"WRITE\(\s*IU_FILE,\s*'([^']*)'\s*\)\s*(.*)", body):
        fmt, args = m.group(1), m.group(2).strip()
        lit = re.match(r"'([^']*)'", args)
        lines.append({"format": fmt, "text": lit.group(1) if lit else None})
        if lit and lit.group(1).startswith("Name,"):
            break
    formats = {}
    for m in re.finditer(r"^\s*(\d+)\s+FORMAT\((.*)\)\s*$", body, re.M):
        formats[m.group(1)] = m.group(2).strip()
    return {"source": "GeosCore/kppsa_interface_mod.F90 (KppSa_Write_Samples)", "header_count_line": "60",
            "lines": lines, "csv_formats": formats}


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GC_REFERENCE_ROOT", "/root/reference")
    layout = extract(os.path.join(root, "GeosCore", "kppsa_interface_mod.F90"))
    out = os.path.join(HERE, "kppsa_layout.json")
    with open(out, "w") as f:
        json.dump(layout, f, indent=1)
    print(out, len(layout["lines"]), "header lines,", len(layout["csv_formats"]), "CSV formats")


if __name__ == "__main__":
    main()
