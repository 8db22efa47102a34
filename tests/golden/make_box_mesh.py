"""Generate tests/golden/box_mesh_hex8/ with the reference's own mesh writer.

Runs the reference's ``python/sfem/mesh/box_mesh.py`` (a hex8 box of 4 x 3 x 3
nodes on [0,2]x[0,1]x[0,1]: 12 elements) where the reference tree is present.
PyYAML is not installed here, so a stand-in ``yaml`` module with a block-style
``dump`` (keys sorted, lists of one-entry maps as ``- key: value``, what PyYAML
writes for these metas) is put on the path for that run; every raw array is the
reference script's own output.

    python tests/golden/make_box_mesh.py REFERENCE_ROOT   (or SFEM_REFERENCE_ROOT set)
"""

import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

def _reference_mesh_dir() -> Path:
    """python/sfem/mesh of the reference tree: the first argument, else $SFEM_REFERENCE_ROOT."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SFEM_REFERENCE_ROOT")
    if not root:
        raise SystemExit("usage: make_box_mesh.py REFERENCE_ROOT (or set SFEM_REFERENCE_ROOT)")
    return Path(root) / "python" / "sfem" / "mesh"


REF = _reference_mesh_dir() if __name__ == "__main__" else None
OUT = Path(__file__).resolve().parent / "box_mesh_hex8"

YAML_STUB = '''
def _fmt(v):
    if isinstance(v, bool):
        return "true" if v else "false"
    return str(v)


def dump(obj, stream=None, **kwargs):
    lines = []
    for k in sorted(obj):
        v = obj[k]
        if isinstance(v, list):
            lines.append(f"{k}:")
            for item in v:
                if isinstance(item, dict):
                    for ik, iv in item.items():
                        lines.append(f"- {ik}: {_fmt(iv)}")
                else:
                    lines.append(f"- {_fmt(item)}")
        else:
            lines.append(f"{k}: {_fmt(v)}")
    text = "\\n".join(lines) + "\\n"
    if stream is None:
        return text
    stream.write(text)


class SafeLoader:
    pass


class CDumper:
    pass


Loader = SafeLoader
Dumper = CDumper
'''


def main():
    assert (REF / "box_mesh.py").exists(), "reference tree unavailable"
    with tempfile.TemporaryDirectory() as tmp:
        stub = Path(tmp) / "stub"
        stub.mkdir()
        (stub / "yaml.py").write_text(YAML_STUB)
        out = Path(tmp) / "mesh"
        env = {"PYTHONPATH": f"{stub}:{REF}", "PATH": "/usr/bin:/bin"}
        subprocess.run([sys.executable, str(REF / "box_mesh.py"), str(out), "-c", "hex8", "-x", "4", "-y", "3",
                        "-z", "3", "--width", "2", "--height", "1", "--depth", "1"], check=True, env=env)
        if OUT.exists():
            shutil.rmtree(OUT)
        shutil.copytree(out, OUT)
    print(sorted(str(p.relative_to(OUT)) for p in OUT.rglob("*")))


if __name__ == "__main__":
    main()
