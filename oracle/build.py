"""Build recipe of the oracle's C restatement (TEST INFRASTRUCTURE ONLY).

``gcc -O3 -fopenmp -shared -fPIC oracle/pdhg_ref.c -o oracle/liboracle_pdhg.so``
(portable flags only: the library is rebuilt on the Arm GPU host).  The
reference itself is pure Python, so nothing of it is compiled here.
"""

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "pdhg_ref.c")
LIB = os.path.join(HERE, "liboracle_pdhg.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle")
    tmp = LIB + ".tmp"
    subprocess.run([cc, "-O3", "-fopenmp", "-shared", "-fPIC", SRC, "-o", tmp, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
