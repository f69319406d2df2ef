"""Verify that every golden value in reference_goldens.json appears verbatim in the cited
Rimu.jl file (run where the reference sources are available):

    python tests/golden/check_goldens.py /path/to/Rimu.jl
"""
import json
import os
import sys


def walk(node, out):
    if isinstance(node, dict):
        if "src" in node and "text" in node:
            out.append((node["src"], node["text"]))
        for v in node.values():
            walk(v, out)
    elif isinstance(node, list):
        for v in node:
            walk(v, out)


def main(root):
    here = os.path.dirname(os.path.abspath(__file__))
    data = json.load(open(os.path.join(here, "reference_goldens.json")))
    items = []
    walk(data, items)
    bad = 0
    for src, text in items:
        path = os.path.join(root, src.split(":")[0])
        body = open(path, encoding="utf-8").read()
        ok = text in body
        bad += not ok
        print(("ok  " if ok else "MISSING ") + src + "  " + text)
    return bad


if __name__ == "__main__":
    sys.exit(main(sys.argv[1]) != 0)
