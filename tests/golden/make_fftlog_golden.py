"""Extract the FFTLog known-answer vectors from the reference's tests.

The reference's ``tests/test_fftlog.py`` (``test_fht_agrees_with_fftlog``) holds four 16-point
outputs of the original Fortran FFTLog program for a(r) = r^(mu+1) exp(-r^2/2),
r = logspace(-4, 4, 16), mu = 0.3: offset 0 and bias 0, then the optimal offset with bias 0,
0.8 and -0.8. This script reads that file as data (the ``theirs = [...]`` literals, in order,
through ``ast``; nothing of it is executed) and writes them to ``fftlog_fortran.json`` beside it.
The reference tree is only needed to regenerate the file.

Usage: python tests/golden/make_fftlog_golden.py <the reference's tests/test_fftlog.py>
"""

from __future__ import annotations

import ast
import json
import sys
from pathlib import Path

OUT = Path(__file__).resolve().parent / "fftlog_fortran.json"


def main(src: Path):
    tree = ast.parse(src.read_text())
    fn = next(n for n in ast.walk(tree) if isinstance(n, ast.FunctionDef) and n.name == "test_fht_agrees_with_fftlog")
    vectors = []
    for node in fn.body:  # top-level statements, in source order
        if isinstance(node, ast.Assign) and any(isinstance(t, ast.Name) and t.id == "theirs" for t in node.targets):
            vectors.append([float(ast.literal_eval(e)) for e in node.value.elts])
    assert len(vectors) == 4 and all(len(v) == 16 for v in vectors), [len(v) for v in vectors]
    cases = [
        {"offset": "zero", "bias": 0.0},
        {"offset": "optimal", "bias": 0.0},
        {"offset": "optimal", "bias": 0.8},
        {"offset": "optimal", "bias": -0.8},
    ]
    doc = {"source": "rocket-fft tests/test_fftlog.py, test_fht_agrees_with_fftlog (Fortran FFTLog output)",
           "input": {"r": "logspace(-4, 4, 16)", "mu": 0.3, "a": "r**(mu+1) * exp(-r**2/2)", "dln": "log(r[1]/r[0])"},
           "cases": [dict(c, out=v) for c, v in zip(cases, vectors)]}
    OUT.write_text(json.dumps(doc, indent=1) + "\n")
    print(f"wrote {OUT}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_fftlog_golden.py <the reference's tests/test_fftlog.py>")
    main(Path(sys.argv[1]))
