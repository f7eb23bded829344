"""Stage the reference's own hot-path modules into oracle/_ref/ -- TEST INFRASTRUCTURE.

The reference is pure Python / PyTorch, so its "build" for this path is its hot-path
modules as they are: this recipe copies them, unmodified, from the reference checkout into
the git-ignored oracle/_ref/ together with a manifest of their SHA-256 digests, so that the
machine that runs bench.py's reference arm (which has no reference checkout) can import and
time the reference's own functions. Nothing under oracle/_ref/ enters this repository's
history. __graft_entry__.build() runs this when the checkout is present.

    python oracle/stage_ref.py [--ref PATH]

load() imports the staged modules under the reference's own module names (they import each
other by those names) and refuses to run if a module of the same name was already imported
from elsewhere in the process (e.g. this package's drop-in modules, installed under the same
names by jscc_recon_spect_cylinder_gb300.install()).
"""
from __future__ import annotations

import argparse
import hashlib
import importlib
import json
import shutil
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_OUT = HERE / "_ref"
DEFAULT_REF = Path("/root/reference")

# the hot-path modules the reference's entry points import (recon loops, sparse projector,
# T builders)
MODULES = ("compton_sparse_ops", "recon_osem_plane", "recon_osem_plane_sparse", "recon_osem_local_cntstat",
           "recon_osem_local_sparse_jsccsd_only", "process_list_plane_strict", "process_list_plane_sparse")


def _sha(p: Path) -> str:
    return hashlib.sha256(p.read_bytes()).hexdigest()


def stage(ref: Path = DEFAULT_REF, out: Path = REF_OUT) -> bool:
    """Copy the modules; False (and nothing written) when the checkout is absent."""
    if not all((ref / f"{m}.py").is_file() for m in MODULES):
        return False
    out.mkdir(parents=True, exist_ok=True)
    manifest = {}
    for m in MODULES:
        src = ref / f"{m}.py"
        shutil.copyfile(src, out / src.name)
        manifest[src.name] = {"sha256": _sha(src), "source": f"{m}.py"}
    (out / "MANIFEST.json").write_text(json.dumps(manifest, indent=1, sort_keys=True))
    return True


def available(out: Path = REF_OUT) -> bool:
    """The staged copies exist and match their manifest."""
    man = out / "MANIFEST.json"
    if not man.is_file():
        return False
    entries = json.loads(man.read_text())
    return all((out / name).is_file() and _sha(out / name) == e["sha256"] for name, e in entries.items()) and \
        all(f"{m}.py" in entries for m in MODULES)


def load(out: Path = REF_OUT) -> dict:
    """{module name: module} of the staged reference modules."""
    if not available(out):
        raise FileNotFoundError(f"the reference's modules are not staged in {out} (run oracle/stage_ref.py)")
    for m in MODULES:
        mod = sys.modules.get(m)
        if mod is not None and Path(getattr(mod, "__file__", "") or "").resolve().parent != out.resolve():
            raise RuntimeError(f"a module named {m!r} is already imported from {getattr(mod, '__file__', None)}; "
                               "the reference's modules must be loaded in a process without it")
    sys.path.insert(0, str(out))
    try:
        return {m: importlib.import_module(m) for m in MODULES}
    finally:
        sys.path.remove(str(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=str(DEFAULT_REF))
    args = ap.parse_args()
    ok = stage(Path(args.ref))
    print(f"staged the reference's modules into {REF_OUT}" if ok else f"no reference checkout at {args.ref}")


if __name__ == "__main__":
    main()
