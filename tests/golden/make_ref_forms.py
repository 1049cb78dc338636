"""Writes tests/golden/ref_forms.json: the element orders the reference's own rsbd8::radixsortcopy
gives on the indexed / offset indirection forms (oracle/ref_forms.cpp, built by
`make -C oracle ref` where the reference header exists).  Run from the repository root:
    python tests/golden/make_ref_forms.py
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
EXE = os.path.join(ROOT, "oracle", "_ref", "ref_forms")


def parse(text: str) -> dict:
    forms = {}
    for line in text.splitlines():
        name, _, rest = line.partition(":")
        if name.startswith("all calls"):
            continue
        forms[name] = [int(x) for x in rest.split()]
    return forms


def main():
    if not os.path.exists(EXE):
        sys.exit("oracle/_ref/ref_forms is not built (make -C oracle ref)")
    out = subprocess.run([EXE], capture_output=True, text=True, check=True).stdout
    data = {"source": "oracle/ref_forms.cpp compiled against Radixsortbidi8.hpp (g++ 13, -std=c++23)",
            "records": "Rec {u64 id; u32 a, b, c, d} x 6: a = 5 3 9 1 7 2, b = 10 60 20 50 30 40, "
                       "c = 6 5 4 3 2 1, d = 1 3 5 2 4 6; id = position",
            "forms": parse(out)}
    with open(os.path.join(HERE, "ref_forms.json"), "w") as f:
        json.dump(data, f, indent=1)


if __name__ == "__main__":
    main()
