"""Place the reference package (ickc/python-autojax) under ``baseline/_ref`` for the reference arm.

    python baseline/stage_reference.py <path of the ickc/python-autojax checkout>

It first tries the offline install

    python -m pip install --no-index --no-build-isolation --find-links /opt/wheelhouse \\
        --target baseline/_ref <checkout>

which needs the reference's build backend (poetry-core).  Where that backend is
not available, it places the package's pure-Python modules under
``baseline/_ref/autojax/`` unchanged, as the install would have.  Either way
``baseline/_ref`` is not committed; it travels with the working tree to the
machine that runs ``bench.py --impl reference``.
"""

from __future__ import annotations

import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
TARGET = HERE / "_ref"
MODULES = ("__init__.py", "numba.py", "original.py")


def main(checkout: str) -> int:
    src = Path(checkout).resolve()
    pkg = src / "src" / "autojax"
    if not (pkg / "numba.py").exists():
        sys.exit(f"{pkg / 'numba.py'} not found")
    TARGET.mkdir(parents=True, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        # the build may write into its source tree, which can be read-only
        copy = Path(tmp) / "src"
        shutil.copytree(src, copy, ignore=shutil.ignore_patterns(".git", ".pixi"))
        r = subprocess.run([sys.executable, "-m", "pip", "install", "--no-index", "--no-build-isolation",
                            "--find-links", "/opt/wheelhouse", "--no-deps", "--target", str(TARGET), str(copy)],
                           capture_output=True, text=True)
    if r.returncode == 0 and (TARGET / "autojax" / "numba.py").exists():
        print("installed with pip")
        return 0
    print("pip install failed (" + (r.stderr.strip().splitlines() or ["?"])[-1] + "); placing the modules")
    dst = TARGET / "autojax"
    dst.mkdir(parents=True, exist_ok=True)
    for name in MODULES:
        shutil.copy2(pkg / name, dst / name)
    (TARGET / "SOURCE").write_text(f"{src}\n")
    print(f"placed {', '.join(MODULES)} in {dst}")
    return 0


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: stage_reference.py <path of the ickc/python-autojax checkout>")
    sys.exit(main(sys.argv[1]))
