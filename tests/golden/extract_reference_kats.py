"""Re-derive the numeric known-answer tests in reference_kat.json from the
reference crate's own test sources (read as text; nothing of the reference is
compiled or run) and check them against the committed fixture.

    python tests/golden/extract_reference_kats.py <reference checkout> [--write]

Covered: solve_linear_system (src/sift.rs:1424-1454), get_gauss_pixel_bilinear
(src/sift.rs:1456-1525), the uniform and gradient images of
tests/integration_test.rs:166-226. The property-style entries (keypoint
ranges, determinism, contrast monotonicity) are statements, not numbers, and
are kept as transcribed. Exits non-zero when the fixture and the sources
disagree.
"""
import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
FIXTURE = HERE / "reference_kat.json"


def _fn_body(src: str, name: str) -> str:
    i = src.index(f"fn {name}(")
    j = src.find("\n    #[test]", i)
    k = src.find("\n#[test]", i)
    ends = [e for e in (j, k) if e > 0]
    return src[i: min(ends) if ends else len(src)]


def _num_list(s: str):
    return json.loads(s.replace(" ", ""))


def extract(ref: Path) -> dict:
    sift = (ref / "src" / "sift.rs").read_text()
    integ = (ref / "tests" / "integration_test.rs").read_text()
    out = {}
    body = _fn_body(sift, "test_solve_linear_system_solvable")
    a = _num_list(re.search(r"let a2 = (\[\[.*?\]\]);", body).group(1))
    b = _num_list(re.search(r"let b2 = (\[.*?\]);", body).group(1))
    x = _num_list(re.search(r"let expected2 = (\[.*?\]);", body).group(1))
    tol = float(re.search(r"\.abs\(\) < ([0-9.e-]+)", body).group(1))
    body = _fn_body(sift, "test_solve_linear_system_singular")
    a2 = _num_list(re.search(r"let a = (\[\[.*?\]\]);", body).group(1))
    b2 = _num_list(re.search(r"let b = (\[.*?\]);", body).group(1))
    out["solve_linear_system"] = [
        {"a": a, "b": b, "x": x, "tol": tol},
        {"a": a2, "b": b2, "x": None},
    ]
    body = _fn_body(sift, "test_get_gauss_pixel_bilinear")
    m = re.search(r"GrayImage::from_raw\((\d+), (\d+), vec!\[([0-9, ]+)\]\)", body)
    w, h = int(m.group(1)), int(m.group(2))
    px = [int(v) for v in m.group(3).split(",")]
    cases, tols = [], set()
    for cm in re.finditer(r"val_at\(([-0-9.]+), ([-0-9.]+)\) - pixel_val\((\d+)\)\)\s*\.abs\(\)\s*<\s*([0-9.e-]+)", body):
        cases.append({"x": float(cm.group(1)), "y": float(cm.group(2)), "v": int(cm.group(3))})
        tols.add(float(cm.group(4)))
    out["get_gauss_pixel_bilinear"] = {
        "image": [px[r * w:(r + 1) * w] for r in range(h)],
        "tol": tols.pop() if len(tols) == 1 else sorted(tols),
        "cases": cases,
    }
    body = _fn_body(integ, "test_sift_on_no_feature_image")
    out["uniform_image"] = {
        "width": int(re.search(r"let width = (\d+);", body).group(1)),
        "height": int(re.search(r"let height = (\d+);", body).group(1)),
        "value": int(re.search(r"Luma\(\[(\d+)u8\]\)", body).group(1)),
        "keypoints": 0,
    }
    body = _fn_body(integ, "test_sift_on_small_image")
    out["small_gradient"] = {
        "width": int(re.search(r"let width = (\d+);", body).group(1)),
        "height": int(re.search(r"let height = (\d+);", body).group(1)),
        "pixel": re.search(r"Luma\(\[\((.*?)\) as u8\]\)", body).group(1),
    }
    return out


def main() -> int:
    if len(sys.argv) < 2:
        print(__doc__)
        return 2
    got = extract(Path(sys.argv[1]))
    fixture = json.loads(FIXTURE.read_text())
    bad = []
    for key, val in got.items():
        have = {k: v for k, v in fixture[key].items() if k != "cite"} if isinstance(fixture[key], dict) else [
            {k: v for k, v in e.items() if k != "cite"} for e in fixture[key]]
        if have != val:
            bad.append(key)
            if "--write" in sys.argv:
                if isinstance(fixture[key], dict):
                    fixture[key].update(val)
                else:
                    for e, v in zip(fixture[key], val):
                        e.update(v)
    if bad and "--write" in sys.argv:
        FIXTURE.write_text(json.dumps(fixture, indent=1) + "\n")
        print("rewrote", ", ".join(bad))
        return 0
    for key in got:
        print(f"{key}: {'MISMATCH' if key in bad else 'matches the reference sources'}")
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main())
