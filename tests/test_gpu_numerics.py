"""The arithmetic the kernels form themselves instead of calling the CUDA
library, checked against the hardware and library operations on the device:
the FMA-corrected quotient that gives the FP64 path the reference's own
u = dist / h, the integer rounding of the FP64 kernel value to float, and the
integer float -> double conversion of the octree walk.  Bit-exact."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_kernel_arithmetic_matches_hardware(seed):
    from timothy_gb300 import session as S

    bad = S.check_numerics(1 << 24, seed)
    assert bad == {"quotient": 0, "round_to_float": 0, "float_to_double": 0}
