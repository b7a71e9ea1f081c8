"""CPU oracle of the BEM hot path -- test infrastructure only (see port.py)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_dir():
    """Directory of the reference's sources, or None where they are absent
    (the GPU machine).  The location is resolved by oracle/build_ref.sh --where
    (its argument, $BEM3_REFERENCE_DIR, or the container's mount)."""
    r = subprocess.run([os.path.join(HERE, "build_ref.sh"), "--where"], capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 and r.stdout.strip() else None
