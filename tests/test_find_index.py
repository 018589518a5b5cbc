"""OctantArray.findIndex / QuadrantArray.findIndex (TMR.pyx, over
TMROctantArray::contains, TMROctant.cpp:404-424): host-side searches of a
forest's arrays, checked here on arrays built directly."""
import numpy as np

from tmr_gb300 import TMR


def test_octant_array_find_index():
    a = np.array([[0, 0, 0, 0, 0, 2, 0],
                  [0, 1 << 28, 0, 0, 1, 2, 0],
                  [1, 0, 1 << 29, 0, 2, 1, 0]], np.intc)
    arr = TMR.OctantArray(a)
    assert arr.findIndex(TMR.Octant(0, 1 << 28, 0, 0, level=2)) == 1
    assert arr.findIndex(TMR.Octant(1, 0, 1 << 29, 0, level=1)) == 2
    assert arr.findIndex(TMR.Octant(1, 0, 1 << 29, 0, level=3)) is None
    assert arr.findIndex(TMR.Octant(1, 0, 1 << 29, 0, level=3), use_nodes=True) == 2
    assert arr.findIndex(TMR.Octant(2, 0, 0, 0, level=0)) is None


def test_quadrant_array_find_index():
    a = np.array([[0, 0, 0, 0, 1, 0],
                  [0, 1 << 29, 0, 1, 1, 0],
                  [3, 0, 1 << 29, 2, 1, 0]], np.intc)
    arr = TMR.QuadrantArray(a)
    assert arr.findIndex(TMR.Quadrant(0, 1 << 29, 0, level=1)) == 1
    assert arr.findIndex(TMR.Quadrant(3, 0, 1 << 29, level=2)) is None
    assert arr.findIndex(TMR.Quadrant(3, 0, 1 << 29, level=2), use_nodes=True) == 2
