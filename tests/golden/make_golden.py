"""Generate golden fixtures from the reference's own data files.

Runs only where the reference tree is mounted (read-only); its output,
tests/golden/reference_data.json, is committed so that tests on machines
without the reference can use it.

Sources (paths inside the reference project):
  data/phantoms/icrp/AM/AM_media.dat   ICRP adult-male media, mass % for
                                       Z = 1,6,7,8,11,12,15,16,17,19,20,26,53
                                       (column list as parsed at
                                       src/libopendxmc/icrpphantomimportpipeline.cpp:157)
  data/phantoms/other/media.dat        same layout, row 53 is Water
  data/bowtiefilters/bowtiefilters.json           {filters: [{name, filterdata: [{angle, weight}]}]}
  data/bowtiefilters/bowtiefilters.json.template  same layout (body W3 120 kV)
  src/libopendxmc/hdf5wrapper.cpp      the study file layout: root dataset names of
                                       HDF5Wrapper::save(DataContainer), and per beam kind
                                       the /beams/<Kind>Beams group and its attribute names
                                       and types (read from the source text)
"""
import json
import os
import re
import sys
from pathlib import Path

# the reference project root: first argument, else $OPENDXMC_REFERENCE, else a checkout
# named "reference" beside this repository
REF = Path(sys.argv[1] if len(sys.argv) > 1 else
           os.environ.get("OPENDXMC_REFERENCE") or Path(__file__).resolve().parents[3] / "reference")
OUT = Path(__file__).resolve().parent / "reference_data.json"
ZS = [1, 6, 7, 8, 11, 12, 15, 16, 17, 19, 20, 26, 53]


def parse_media(path: Path) -> dict:
    """Rows: '<id> <name ...> <13 mass percentages>'; header lines are skipped."""
    media = {}
    for line in path.read_text(errors="replace").splitlines():
        m = re.match(r"^\s*(\d+)\s+(.*)$", line)
        if not m:
            continue
        tokens = m.group(2).split()
        if len(tokens) < 14:
            continue
        try:
            vals = [float(x) for x in tokens[-13:]]
        except ValueError:
            continue
        name = " ".join(tokens[:-13])
        media[int(m.group(1))] = {"name": name, "composition": {str(z): v for z, v in zip(ZS, vals) if v > 0}}
    return media


def parse_bowties(path: Path) -> dict:
    doc = json.loads(path.read_text())
    out = {}
    for f in doc.get("filters", []):
        data = [[d["angle"], d["weight"]] for d in f.get("filterdata", []) if "angle" in d and "weight" in d]
        if data and f.get("name"):
            out[f["name"]] = data
    return out


def parse_hdf5_layout(path: Path) -> dict:
    """Dataset names of the study save and, per beam save function, its group kind and
    its attributes with their element type."""
    src = path.read_text(errors="replace")
    funcs = re.split(r"\nbool HDF5Wrapper::save\(", src)
    datasets, beams = [], {}
    for f in funcs[1:]:
        head = f.split(")", 1)[0]
        if "DataContainer" in head:
            datasets = re.findall(r'names\[0\] = "(\w+)";', f.split("\n}\n", 1)[0])
            continue
        m = re.search(r'"/beams/(\w+)/1"', f)
        if not m:
            continue
        body = f.split("\n}\n", 1)[0]
        attrs = {}
        for t, name in re.findall(r'saveAttribute<([\w:]+)>\(beamgroup, "(\w+)"', body):
            attrs[name] = "uint64" if "uint64" in t else "double"
        beams[m.group(1)] = attrs
    return {"datasets": datasets, "beams": beams}


def main():
    res = {
        "AM_media": parse_media(REF / "data/phantoms/icrp/AM/AM_media.dat"),
        "other_media": parse_media(REF / "data/phantoms/other/media.dat"),
        "bowtiefilters": parse_bowties(REF / "data/bowtiefilters/bowtiefilters.json"),
        "bowtie_template": parse_bowties(REF / "data/bowtiefilters/bowtiefilters.json.template"),
        "hdf5_layout": parse_hdf5_layout(REF / "src/libopendxmc/hdf5wrapper.cpp"),
    }
    OUT.write_text(json.dumps(res, indent=1, sort_keys=True))
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes): {len(res['AM_media'])} AM media, "
          f"{len(res['bowtiefilters'])} bowtie filters")


if __name__ == "__main__":
    main()
