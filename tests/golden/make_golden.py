"""Generate tests/golden/torch_cases.json.

The reference pins its direct convolution and its padding against LibTorch
(src/conv/tests.rs:36-547 via tch conv1d/2d/3d; src/padding/mod.rs:763-861
via tch f_pad).  tch cannot be built here, so this script recomputes the
same expected values with torch.nn.functional on the same literal inputs,
calling torch exactly the way each reference test calls tch (kernel flipped
where the reference test flips it).  Run:  python tests/golden/make_golden.py
"""
import json
import os

import torch
import torch.nn.functional as F

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "torch_cases.json")


def t(a):
    x = torch.tensor(a, dtype=torch.float64)
    return x.reshape((1, 1) + tuple(x.shape))


def run_conv(nd, arr, ker, flip, **kw):
    fn = {1: F.conv1d, 2: F.conv2d, 3: F.conv3d}[nd]
    k = t(ker)
    if flip:
        k = torch.flip(k, dims=list(range(2, 2 + nd)))
    y = fn(t(arr), k, **kw)
    return torch.round(y[0, 0]).to(torch.int64).tolist()


def conv_cases():
    # name, arr, kernel, dilation, reverse, conv_mode, torch call (kernel
    # flipped for torch when the reference test flips it)
    C = []

    def add(name, nd, arr, ker, dil, rev, mode, flip, **kw):
        C.append({"name": name, "arr": arr, "kernel": ker, "dilation": dil, "reverse": rev,
                  "mode": mode, "expected": run_conv(nd, arr, ker, flip, **kw),
                  "source": "src/conv/tests.rs"})

    # Full mode (src/conv/tests.rs:44-114)
    add("full_1d", 1, [1, 2, 3, 4, 5], [1, 2, 1], 1, True, ["Full"], False, padding=2)
    add("full_2d", 2, [[1, 2], [3, 4]], [[1, 1], [1, 1]], 1, True, ["Full"], False, padding=1)
    add("full_3d", 3, [[[1, 2]], [[3, 4]]], [[[1, 1]], [[1, 1]]], 1, True, ["Full"], False,
        padding=(1, 0, 1))
    # Same mode (:120-201)
    add("same_1d", 1, [1, 2, 3, 4, 5], [1, 2, 1], 1, True, ["Same"], False, padding="same")
    add("same_2d", 2, [[1, 2, 3], [4, 5, 6], [7, 8, 9]], [[1, 0, -1], [2, 0, -2], [1, 0, -1]], 1,
        True, ["Same"], True, padding="same")
    add("same_3d", 3, [[[1, 2, 3]], [[4, 5, 6]]], [[[1, 1, 1]]], 1, True, ["Same"], False,
        padding="same")
    # Valid mode (:207-274)
    add("valid_1d", 1, [1, 2, 3, 4, 5], [1, 2, 1], 1, True, ["Valid"], False, padding="valid")
    add("valid_2d", 2, [[1, 2, 3], [4, 5, 6], [7, 8, 9]], [[1, 1], [1, 1]], 1, True, ["Valid"],
        False, padding="valid")
    add("valid_3d", 3, [[[1, 2, 3], [4, 5, 6]], [[7, 8, 9], [10, 11, 12]]], [[[1, 1]], [[1, 1]]],
        1, True, ["Valid"], False, padding="valid")
    # Strides (:280-364)
    add("stride_2_1d", 1, [1, 2, 3, 4, 5, 6], [1, 1, 1], 1, True, ["Custom", [1], [2]], False,
        stride=2, padding=1)
    add("stride_2_2d", 2, [[1, 2, 3, 4], [5, 6, 7, 8], [9, 10, 11, 12]], [[1, 1], [1, 1]], 1, True,
        ["Custom", [1, 1], [2, 2]], False, stride=(2, 2), padding=1)
    add("stride_3_1d", 1, [1, 2, 3, 4, 5, 6, 7, 8, 9], [1, 2, 1], 1, True, ["Custom", [2], [3]],
        False, stride=3, padding=2)
    # Dilation (:370-460), no_reverse against torch's cross-correlation
    add("dilation_2_1d", 1, [1, 2, 3, 4, 5, 6], [1, 1, 2], 2, False, ["Custom", [4], [2]], False,
        stride=2, padding=4, dilation=2)
    add("dilation_2_2d", 2, [[1, 1, 1], [1, 1, 1], [1, 1, 2]], [[2, 1, 1], [1, 1, 1]], 2, False,
        ["Same"], False, padding="same", dilation=2)
    add("dilation_2_3d", 3, [[[1, 2], [3, 4]], [[5, 6], [7, 8]]],
        [[[1, 1, 1], [1, 1, 1], [1, 1, 1]], [[1, 1, 1], [1, 1, 1], [1, 1, 1]]], 2, False,
        ["Custom", [2, 2, 2], [1, 2, 1]], False, stride=(1, 2, 1), padding=2, dilation=2)
    # Kernel reversal (:466-547)
    add("with_reverse", 1, [1, 2, 3, 4, 5, 6], [1, 1, 2], 2, True, ["Custom", [4], [2]], True,
        stride=2, padding=4, dilation=2)
    add("no_reverse", 1, [1, 2, 3, 4, 5, 6], [1, 1, 2], 2, False, ["Custom", [4], [2]], False,
        stride=2, padding=4, dilation=2)
    return C


def pad_cases():
    # aligned_with_libtorch (src/padding/mod.rs:763-801): Same/Full-unfolded
    # pads, modes checked against torch pad on the same arrays
    C = []
    arrs = [
        ("3d_same_k333", [[[1, 2, 3], [3, 4, 5]], [[5, 6, 7], [7, 8, 9]]], [[1, 1], [1, 1], [1, 1]]),
        ("2d_full_k22", [[1, 2], [3, 4]], [[1, 1], [1, 1]]),
        ("1d_same_k4", [1, 2, 3], [[2, 1]]),
    ]
    for name, arr, pads in arrs:
        x = t(arr)
        flat = []
        for p in reversed(pads):  # torch pads last axis first
            flat += [p[0], p[1]]
        for mode, tmode, val in [("Zeros", "constant", 0.0), ("Const", "constant", 7.0),
                                 ("Replicate", "replicate", None), ("Reflect", "reflect", None),
                                 ("Circular", "circular", None)]:
            if val is None:
                y = F.pad(x, flat, mode=tmode)
            else:
                y = F.pad(x, flat, mode=tmode, value=val)
            C.append({"name": f"{name}_{mode}", "arr": arr, "pads": pads, "mode": mode,
                      "const": 7 if mode == "Const" else 0,
                      "expected": torch.round(y[0, 0]).to(torch.int64).tolist(),
                      "source": "src/padding/mod.rs:763-801"})
    return C


if __name__ == "__main__":
    doc = {
        "generator": "tests/golden/make_golden.py",
        "torch": torch.__version__,
        "conv": conv_cases(),
        "padding": pad_cases(),
    }
    with open(OUT, "w") as f:
        json.dump(doc, f, indent=1)
    print(f"wrote {OUT}: {len(doc['conv'])} conv, {len(doc['padding'])} padding cases")
