"""setup(..., unaligned_anisotropic=True) behaves as the reference's does.

The reference's unaligned-anisotropic mode splits each voxel's heat balance into 15 ADI stages
(alternatingdirection_c_pyx.pyx:511-564), but its adi_setup builds three stage matrices (pyx:418-445), so the
stage-count assertion in add_equation_to_adi_matrices (pyx:452) fails at the first voxel of every problem.
tests/golden/unaligned_anisotropic.json records what the reference raised on three problems (a diagonal tensor,
an off-diagonal tensor, the scalar-k mixed grid with fixed voxels); this implementation raises the same
exception type on the same problems, after validating the classes, and runs the aligned problems normally with
the flag off.  No GPU is needed: the error comes before anything is compiled on the device.
"""
import json
import os

import pytest

from conftest import GOLDEN
import heatsim2_gb300 as hs
from heatsim2_gb300 import workloads as W

with open(os.path.join(GOLDEN, "unaligned_anisotropic.json")) as _fh:
    RECORDED = json.load(_fh)


def _spec(label):
    if label == "scalar_k":
        return W.mixed_small()
    spec = W.line_grid((3, 4, 5))
    spec["boundaries"][0] = ["conducting_anisotropic"]
    spec["materials"][0][1] = ([[5.0, 0, 0], [0, 4.0, 0], [0, 0, 3.0]] if label == "aligned_tensor"
                               else [[5.0, 0.3, 0.0], [0.3, 5.0, 0.0], [0.0, 0.0, 5.0]])
    return spec


@pytest.mark.parametrize("label", sorted(RECORDED))
def test_unaligned_mode_raises_as_the_reference(label):
    rec = RECORDED[label]
    assert rec == {"raised": "AssertionError", "file": "alternatingdirection_c_pyx.pyx", "line": 452}
    with pytest.raises(AssertionError) as info:
        hs.setup(*W.setup_args(hs, _spec(label)), unaligned_anisotropic=True)
    assert "alternatingdirection_c_pyx.pyx:452" in str(info.value)


def test_invalid_classes_are_reported_before_the_mode_error():
    """As in the reference, the classes are evaluated before the stage split: a wrong-dtype class array is a
    ValueError whatever the flag."""
    spec = _spec("aligned_tensor")
    spec["arrays"]["material"] = spec["arrays"]["material"].astype("int32")
    with pytest.raises(ValueError):
        hs.setup(*W.setup_args(hs, spec), unaligned_anisotropic=True)
