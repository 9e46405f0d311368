"""Extract the reference's own test vectors and example inputs into tests/golden/.

The reference's only tests (src/shadertoy.rs:354-453) pin its WGSL text
surgery: `remove_function` (:357-392) and `rename_function` (:394-401).  This
script reads those tests as text from a reference checkout and writes their
inputs and expected facts to wgsl_surgery.json.  It also stores the example
SDF files the reference ships as its inputs (examples/*.sdf3d, *.frag) in
reference_examples.json, so that the GPU tests can mesh them where no
reference checkout exists.  Run from the repository root:

    python tests/golden/make_golden.py /path/to/sdf2mesh
"""
from __future__ import annotations

import json
import os
import re
import sys


def raw_strings(text):
    return re.findall(r'r#"(.*?)"#', text, flags=re.S)


def main(ref_root):
    src = open(os.path.join(ref_root, "src", "shadertoy.rs")).read()
    tests = src[src.index("#[cfg(test)]"):]
    remove_block = tests[tests.index("fn remove_function()"):tests.index("fn rename_function()")]
    rename_block = tests[tests.index("fn rename_function()"):tests.index("fn test_naga()")]
    remove_in = raw_strings(remove_block)[0]
    rename_in = raw_strings(rename_block)[0]
    out = {
        "source": "src/shadertoy.rs:357-401 (WilstonOreo/sdf2mesh)",
        "remove_function": {
            "input": remove_in,
            "steps": [
                {"remove": "fn main_1()", "contains": ["fn mainImage(fragColor"], "absent": ["fn main_1()"]},
                {"remove": "fn main(", "contains": ["fn mainImage(fragColor"], "absent": ["fn main()"]},
                {"remove": "fn mainImage(", "trim_equals": "@fragment"},
            ],
        },
        "rename_function": {
            "input": rename_in, "old": "normal", "new": "sdf3d_normal",
            "contains": ["fn sdf3d_normal(p_4: vec3<f32>, epsilon: f32) -> vec3<f32>"],
        },
    }
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "wgsl_surgery.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    examples = {}
    for name in ("torus.sdf3d", "martin_cube.sdf3d", "p_key.sdf3d", "mandelmesh.frag"):
        with open(os.path.join(ref_root, "examples", name)) as f:
            examples[name] = f.read()
    with open(os.path.join(here, "reference_examples.json"), "w") as f:
        json.dump({"source": "examples/ (WilstonOreo/sdf2mesh), the reference's example inputs",
                   "files": examples}, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("S2M_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout>  (or set S2M_REFERENCE_DIR)")
    main(ref)
