"""Compiles tests/cpp/facade_pile.cpp against the C++20 facade and the in-tree library."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "cpp", "_build")


def build_facade_pile():
    from physkit_gb300 import build

    lib = build.build()
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "facade_pile")
    src = os.path.join(HERE, "cpp", "facade_pile.cpp")
    cmd = ["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           src, "-o", exe, "-L", os.path.dirname(lib), "-lphyskit_gb300", "-Wl,-rpath," + os.path.dirname(lib)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def write_scene(scene, path):
    """Boxes only: the 33-double records facade_pile.cpp reads."""
    import numpy as np

    b = scene.bodies
    rec = np.zeros((len(b), 33))
    rec[:, 0] = b["type"]
    for i, r in enumerate(b):
        sh = scene.shapes[int(r["shape"])]
        assert sh[0] == "box"
        rec[i, 1:4] = sh[1:4]
    rec[:, 4:7] = b["pos"]
    rec[:, 7:11] = b["quat"]
    rec[:, 11:14] = b["vel"]
    rec[:, 14:17] = b["ang_vel"]
    rec[:, 17] = b["mass"]
    rec[:, 21:30] = b["inertia"]
    rec[:, 30] = b["restitution"]
    rec[:, 31] = b["friction"]
    with open(path, "wb") as f:
        f.write(np.int32(len(b)).tobytes())
        f.write(rec.astype("<f8").tobytes())


def read_result(path):
    import numpy as np

    raw = open(path, "rb").read()
    ns = int(np.frombuffer(raw[:4], dtype=np.int32)[0])
    rows = np.frombuffer(raw[4:4 + ns * 14 * 8], dtype="<f8").reshape(ns, 14)
    off = 4 + ns * 14 * 8
    npairs = int(np.frombuffer(raw[off:off + 4], dtype=np.int32)[0])
    pairs = np.frombuffer(raw[off + 4:off + 4 + 8 * npairs], dtype="<u8")
    return rows, pairs
