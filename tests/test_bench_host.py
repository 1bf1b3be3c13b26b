"""Host-side figures of bench.py, on the CPU: the fixed denominators of the roofline.

The algorithmic bytes and FP64 operations per element and RK4 stage follow the reference's
data model (packed inverse stiffnesses, element coefficient blocks, β at the mass points, face
coefficients, the source or manufactured-solution projections and 4.25 state-sized transfers per
stage; the volume, u-equation, trace, lift, face, Chebyshev set-up and RK4 operations plus the
per-step cost of the Chebyshev iteration). Their values are pinned here for four workloads:
the manufactured-solution run (q_u = 3, q_v = 2), the bench's source-mode run (q = 6), the
jumping-coefficient run (q_u = 5, q_v = 4, one-sided faces) and the adjoint's forward run (q = 4).
"""
import json

import pytest

import bench


@pytest.mark.parametrize("nu, nv, qh, one_sided, s_mode, bytes_, flops1, per_step", [
    (4, 3, 4, False, 4, 2866, 3850, 426),          # mms, q_u = 3, q_v = 2 (four Π arrays)
    (7, 7, 10, False, 1, 15556, 23478, 5250),      # source mode, q = 6 (the bench)
    (6, 5, 7, True, 1, 9242, 12922, 1930),         # initial-value mode, q_u = 5, q_v = 4, one-sided faces
    (5, 5, 7, False, 1, 5612, 8890, 1930),         # source mode, q = 4 (the adjoint's forward run)
])
def test_algorithmic_bytes_and_flops(nu, nv, qh, one_sided, s_mode, bytes_, flops1, per_step):
    assert bench.alg_bytes_per_element_stage(nu, nv, qh, one_sided=one_sided, s_mode_nv2=s_mode) == bytes_
    assert bench.alg_flops_per_element_stage(nu, nv, qh, 1) == flops1
    assert bench.alg_flops_per_element_stage(nu, nv, qh, 2) - flops1 == per_step


def test_bench_config_is_the_same_for_both_arms():
    """The `config` of the GPU arm and of the reference arm (the driver compares them)."""
    E = bench.NMESH ** 2
    dof = E * ((bench.Q + 1) ** 2 * 2)
    a = bench.bench_config(E, dof, "front")
    assert a == bench.bench_config(E, dof, "front")
    assert a["elements"] == 262144 and a["dof"] == 25690112
    json.dumps(a)

