"""Extract the reference's known-answer values into reference_goldens.json.

Reads the Rust test modules of QuState/spinoza v0.5.1 as text (it never runs
them: there is no Rust toolchain here) and records, per #[test] function,
every `assert_float_closeness(<array>[<index>], <expected>, <eps>)` and every
numeric array literal (`let vals = [...]`, `let expected_reals = [...]`) with
its file:line.  tests/test_oracle_golden.py restates each test's setup and
checks the oracle (and the GPU path) against these values.

Usage:  python tests/golden/extract_reference_goldens.py <path of a checkout of the reference>
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

FILES = ["spinoza/src/gates.rs", "spinoza/src/core.rs", "spinoza/src/measurement.rs", "spinoza/src/circuit.rs",
         "spinoza/src/math.rs"]

ASSERT = re.compile(r"assert_float_closeness\(\s*([^,]+?)\s*,\s*([-+0-9.eE_]+)\s*,\s*([-+0-9.eE_]+|\w+)\s*\)")
LET_NUM = re.compile(r"let\s+(\w+)\s*=\s*([-+0-9.eE_]+)\s*;")
ARRAY_START = re.compile(r"let\s+(?:mut\s+)?(\w+)\s*(?::[^=]+)?=\s*\[")
FN = re.compile(r"^\s*fn\s+(\w+)\s*\(")
NUM = re.compile(r"-?\d+\.\d+(?:[eE][-+]?\d+)?|-?\d+\.?(?:[eE][-+]?\d+)")


def parse_file(root: Path, rel: str) -> dict:
    text = (root / rel).read_text().splitlines()
    out: dict = {}
    in_tests = False
    current = None
    pending_test = False
    i = 0
    while i < len(text):
        line = text[i]
        lineno = i + 1
        if "#[cfg(test)]" in line:
            in_tests = True
        if in_tests and "#[test]" in line:
            pending_test = True
        m = FN.match(line)
        if in_tests and m:
            name = m.group(1)
            current = name if pending_test else None
            if current:
                out[f"{Path(rel).name}::{current}"] = {"file": rel, "line": lineno, "asserts": [], "arrays": {}}
            pending_test = False
        if current:
            key = f"{Path(rel).name}::{current}"
            lm = LET_NUM.search(line)
            if lm:
                out[key].setdefault("lets", {})[lm.group(1)] = float(lm.group(2).replace("_", ""))
            am = ARRAY_START.search(line)
            if am and "vec!" not in line:
                # collect until the closing bracket
                buf, j = line[am.end():], i
                while "]" not in buf:
                    j += 1
                    buf += " " + text[j]
                body = buf[: buf.index("]")]
                nums = [float(x.replace("_", "")) for x in NUM.findall(body)]
                if nums:
                    out[key]["arrays"][am.group(1)] = {"line": lineno, "values": nums}
            for a in ASSERT.finditer(line):
                target, expected, eps = a.group(1), a.group(2), a.group(3)
                arr = re.match(r"(?:\w+\.)*(\w+)\[(.+)\]$", target.strip())
                out[key]["asserts"].append({
                    "line": lineno,
                    "target": target.strip(),
                    "array": arr.group(1) if arr else None,
                    "index": arr.group(2) if arr else None,
                    "expected": float(expected.replace("_", "")),
                    "eps": float(eps.replace("_", "")) if re.match(r"[-+0-9.]", eps)
                    else out[key].get("lets", {})[eps],
                })
        i += 1
    return {k: v for k, v in out.items() if v["asserts"] or v["arrays"]}


def main() -> None:
    if len(sys.argv) < 2:
        sys.exit("usage: extract_reference_goldens.py <path of a checkout of the reference repository>")
    root = Path(sys.argv[1])
    goldens = {"source": "QuState/spinoza v0.5.1 (spinoza/Cargo.toml:3), Rust #[test] modules",
               "extracted_by": "tests/golden/extract_reference_goldens.py", "tests": {}}
    for rel in FILES:
        goldens["tests"].update(parse_file(root, rel))
    dst = Path(__file__).with_name("reference_goldens.json")
    dst.write_text(json.dumps(goldens, indent=1) + "\n")
    print(f"wrote {dst} with {len(goldens['tests'])} tests")


if __name__ == "__main__":
    main()
