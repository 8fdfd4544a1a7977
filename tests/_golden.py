"""Loading helpers for the golden vectors produced by tests/golden/make_golden.py."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(tag: str, name: str):
    return np.load(os.path.join(GOLDEN, tag, name + ".npz"))


def meta(tag: str) -> dict:
    z = load(tag, "init")
    return {str(k): float(v) for k, v in zip(z["meta_keys"], z["meta_vals"])}


TAGS = {"kat-small-fd": ("kat-small.job", 0), "kat-small-nsfd": ("kat-small-nsfd.job", 1)}

# Jobs with an initial state and a 12-step march of the reference, for layout edge cases.
LAYOUT_TAGS = {"kat-small-ragged": ("kat-small-ragged.job", 0)}

# Jobs with only an initial state and a 12-step march of the reference (no single-stage vectors):
# the TF/SF seed, the external laser fields and the optical undulator.
BEAM_TAGS = {"kat-small-seed": ("kat-small-seed.job", 1), "kat-small-ext": ("kat-small-ext.job", 0),
             "kat-small-optical": ("kat-small-optical.job", 0)}
