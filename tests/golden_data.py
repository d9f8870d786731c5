"""Loaders for the golden fixtures made by tests/golden/make_fixtures.py."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def w_loop():
    """The testD2BI input (27,847 W atoms), the shipped image and its header."""
    inp = np.load(os.path.join(GOLDEN, "w_loop_input.npz"))
    dat = np.load(os.path.join(GOLDEN, "w_loop_dat.npz"))
    hdr = json.loads(str(dat["header"]))
    box = inp["box"]
    return {
        "pos": inp["pos"],
        "a_super": np.diag(box[:, 1] - box[:, 0]),
        "img": dat["img"],
        "header": hdr,
        # the header's rotation is matmul(R, U), written column-major
        "RU": np.array(hdr["rotation"]).reshape(3, 3).T,
        "d": hdr["img space (A)"],
        "xi0": hdr["xi (A)"][0],
        "xig": hdr["xi (A)"][1],
        "png": np.load(os.path.join(GOLDEN, "w_loop_png.npz"))["levels"],
    }


def linkcell_kat():
    with open(os.path.join(GOLDEN, "linkcell_kat.json")) as f:
        return json.load(f)


def electrons_kat():
    with open(os.path.join(GOLDEN, "electrons_kat.json")) as f:
        return json.load(f)
