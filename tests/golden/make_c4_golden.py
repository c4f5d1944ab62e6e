"""Generate tests/golden/connect_four.json from the REFERENCE's own
connect-four known answer: its base board (src/test_suite/connect_four/
board.txt, read the way scan_board in connect_four.h:89-104 reads it: '.'
empty, 'o' human, 'x' computer, other characters skipped), the default
look-ahead (DEFINE_int32(maxlevel, ...) in connect_four.h) and the move
values its check_persistent_task compares against (connect_four.h:344-351).

Run from the repository root with the reference present:
    python tests/golden/make_c4_golden.py
"""
from __future__ import annotations

import json
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "connect_four.json")


def main() -> None:
    sys.path.insert(0, ROOT)
    from oracle.build_ref import reference_root
    root = reference_root()
    if root is None:
        raise SystemExit("reference checkout not found (set WGM_REFERENCE_ROOT)")
    REF = os.path.join(root, "src", "test_suite", "connect_four")
    cells = []
    with open(os.path.join(REF, "board.txt")) as f:
        for ch in f.read():
            if ch in ".ox":
                cells.append(".ox".index(ch))
            if len(cells) == 42:
                break
    header = open(os.path.join(REF, "connect_four.h")).read()
    maxlevel = int(re.search(r"DEFINE_int32\(maxlevel,\s*(\d+)", header).group(1))
    consts = {"PLUS_INF": 666, "MINUS_INF": -666}
    want = {}
    for i, v in re.findall(r"h_next_move_value\[(\d)\] == \(cl_int\)([A-Z_0-9-]+)", header):
        want[int(i)] = consts[v] if v in consts else int(v)
    assert len(cells) == 42 and sorted(want) == list(range(7))
    with open(OUT, "w") as f:
        json.dump({"board": cells, "maxlevel": maxlevel,
                   "next_move_value": [want[i] for i in range(7)],
                   "source": "test_suite/connect_four/board.txt; connect_four.h:14,344-351"},
                  f, indent=1)
    print(OUT, maxlevel, [want[i] for i in range(7)])


if __name__ == "__main__":
    main()
