"""Stages the Hydra headers a translation unit can reach into a copy of the source tree layout.

Test infrastructure (called by oracle/build_ref.sh): the copy lets the reference harness be built
on a machine that has the staged headers but not the Hydra tree.  The starting set is what the
compiler reports it opened (DEPS, `g++ -M` output: it resolves includes whose names come from
macros), and every #include line of those files is followed as well, whatever #if surrounds it
(the compiler's list omits a header whose `#pragma once` it matched to an identical file already
read).  Headers outside the tree (the C++ library, OpenMP) are left to the compiler.

    python stage_ref_headers.py SRC_TREE OUT_DIR ENTRY.cpp [DEPS ...]
"""
from __future__ import annotations

import re
import shutil
import sys
from pathlib import Path

INCLUDE = re.compile(r'^\s*#\s*include\s*([<"])([^>"]+)[>"]', re.M)


def closure(src: Path, entries: list[Path]) -> set[Path]:
    seen: set[Path] = {e for e in entries if src in e.parents}
    todo = list(entries)
    while todo:
        f = todo.pop()
        try:
            text = f.read_text(errors="replace")
        except OSError:
            continue
        for kind, name in INCLUDE.findall(text):
            cands = ([f.parent / name] if kind == '"' else []) + [src / name]
            for c in cands:
                c = Path(c).resolve()
                if c.is_file() and src in c.parents:
                    if c not in seen:
                        seen.add(c)
                        todo.append(c)
                    break
    return seen


def main(argv):
    src, out = Path(argv[1]).resolve(), Path(argv[2])
    entries = [Path(argv[3]).resolve()]
    for deps in argv[4:]:
        for tok in Path(deps).read_text().replace("\\\n", " ").split():
            p = Path(tok)
            if p.is_file():
                entries.append(p.resolve())
    files = closure(src, entries)
    for f in sorted(files):
        dst = out / f.relative_to(src)
        dst.parent.mkdir(parents=True, exist_ok=True)
        shutil.copy2(f, dst)
    print(f"stage_ref_headers: {len(files)} headers into {out}")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
