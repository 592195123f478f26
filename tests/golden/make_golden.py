"""Extracts the reference's golden vectors for the hot path into JSON fixtures.

Run where a checkout of the reference (BlueBrain/Livre) is available:
    python tests/golden/make_golden.py <path to the Livre source tree>
(or set LIVRE_SOURCE_DIR). It reads, as text:
  - tests/data/lodSelection.cpp:70-207  (getVisibles cases and expected ids)
  - tests/core/tf_f.1dt                 (transfer-function file of
                                          tests/core/transferFunction.cpp:53-62)
  - tests/data/nucleon.raw              (41^3 uint8 volume, raw:// fixture)
and writes lod_selection.json, tf_f.json and nucleon.raw beside this script.
Nothing at test time reads the reference tree.
"""
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def lod_cases(src):
    text = open(src).read()
    # volume URI
    uri = re.search(r'lunchbox::URI uri\("([^"]+)"\)', text).group(1)
    # projection / modelview arrays inside getVisibles
    proj = re.search(r"projArray\[\] = \{([^}]*)\}", text).group(1)
    mv = re.search(r"mvArray\[\] = \{([^}]*)\}", text).group(1)
    nums = lambda s: [float(x) for x in re.findall(r"-?\d+\.?\d*(?:e-?\d+)?", s)]
    cases = []
    body = text[text.index("BOOST_AUTO_TEST_CASE(testLODSelection)"):]
    # each block: getVisibles(dataSource, H, sse, minLOD, maxLOD) ... results = {...}
    pat = re.compile(
        r"(?:const uint32_t maxMinLevel = (\d+);\s*)?const Identifiers& visibles =\s*"
        r"getVisibles\(dataSource,\s*(\d+),\s*([\d.]+),\s*(\w+),\s*(\w+)\);\s*"
        r"const Identifiers results = \{([^}]*)\}", re.S)
    for m in pat.finditer(body):
        mml = m.group(1)
        def val(tok):
            return int(mml) if tok == "maxMinLevel" else int(tok)
        cases.append({
            "window_height": int(m.group(2)), "sse": float(m.group(3)),
            "min_lod": val(m.group(4)), "max_lod": val(m.group(5)),
            "expected": [int(x) for x in re.findall(r"\d+", m.group(6))]})
    return {"uri": uri, "proj": nums(proj), "mv": nums(mv), "cases": cases,
            "source": "tests/data/lodSelection.cpp:38-207"}


def tf_file(src):
    toks = open(src).read().split()
    n = int(toks[0])
    vals = [float(x) for x in toks[1:1 + 4 * n]]
    return {"n": n, "rgba": vals, "source": "tests/core/tf_f.1dt"}


def main(ref):
    out = lod_cases(os.path.join(ref, "tests/data/lodSelection.cpp"))
    assert len(out["cases"]) == 8, len(out["cases"])
    json.dump(out, open(os.path.join(HERE, "lod_selection.json"), "w"), indent=1)
    json.dump(tf_file(os.path.join(ref, "tests/core/tf_f.1dt")),
              open(os.path.join(HERE, "tf_f.json"), "w"))
    shutil.copyfile(os.path.join(ref, "tests/data/nucleon.raw"),
                    os.path.join(HERE, "nucleon.raw"))
    print("wrote", len(out["cases"]), "lod cases")


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LIVRE_SOURCE_DIR")
    if not src:
        sys.exit("usage: make_golden.py <Livre source tree> (or set LIVRE_SOURCE_DIR)")
    main(src)
