"""Copy the reference project's own test fixtures for this path into tests/golden.

The reference pins its renderer with 96x96 regression PNGs rendered from small
`.ft` scenes (crates/forgedthoughts/tests/render_regression.rs:27-107) and its
front-end with parse/eval error fixtures (crates/forgedthoughts/tests/
golden.rs:9-53).  Machines that run the tests have no copy of the reference, so the fixtures
travel with the tests.  Run from the repository root:

    python tests/golden/make_reference_fixtures.py /path/to/reference
"""
import shutil
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def main(reference: str) -> None:
    src = Path(reference) / "crates" / "forgedthoughts" / "tests" / "fixtures"
    for sub in ("render_regression", "parse_err", "eval_err"):
        dst = HERE / "reference_fixtures" / sub
        dst.mkdir(parents=True, exist_ok=True)
        for f in sorted((src / sub).iterdir()):
            if f.suffix in (".ft", ".png", ".err"):
                shutil.copyfile(f, dst / f.name)
                print(dst / f.name)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_reference_fixtures.py <path to the reference project>")
    main(sys.argv[1])
