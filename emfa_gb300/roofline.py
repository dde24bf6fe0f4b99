"""FLOP and byte models of the hot path: the one definition that the bench's
roofline numbers and the design notes use.

Counts are algorithmic: the work the formulation requires, not what a
kernel happens to execute (a split-FP16 residual does three tensor products
but is credited with one complex product).
"""
from __future__ import annotations


def block_product_flops(n: int, nrhs: int) -> float:
    """Complex N x N times N x R: 8 real FLOP per complex multiply-add."""
    return 8.0 * n * n * nrhs


def split_fp16_inner_bytes(n: int, nrhs: int) -> float:
    """Inner product of the mixed solver: the FP16 hi plane of Z (n x 2n
    halves), the packed FP16 right-hand sides (2R rows of 2n halves) and the
    complex64 output."""
    return 2.0 * n * 2 * n + 2.0 * (2 * nrhs) * (2 * n) + 8.0 * n * nrhs


# DRAM bytes (read + write) of one launch of the split-FP16 inner product at
# n = 7680, R = 360, from an ncu capture of that kernel at that size (one
# pass); the algorithmic figure is split_fp16_inner_bytes(7680, 360).
INNER_TRAFFIC_7680x360 = 261.3e6


def fp32_nominal_tflops(sm_count: int = 152, sm_mhz: float = 2070.0) -> float:
    """Nominal FP32 FMA rate: 128 lanes per SM, 2 FLOP per FMA."""
    return sm_count * 128 * 2 * sm_mhz * 1e6 / 1e12


def fill_flops(n_tri: int, cfie: bool) -> float:
    """Regular-pair fill counted per unique triangle pair: 9 point pairs per
    pair, 75 FLOP per point pair for CFIE and 40 for EFIE (sqrt, sin, cos
    and reciprocal counted as 2 each)."""
    return float(n_tri) * n_tri * 9 * (75 if cfie else 40)


def fill_bytes(n: int, fp64: bool = False) -> float:
    """Writing Z once."""
    return float(n) * n * (16 if fp64 else 8)


def mlfma_matvec_bytes(n: int, nnz: int, level_boxes, poles, comps: int = 3, near_index_bytes: int = 0,
                       radrec_comps: int | None = None) -> float:
    """Compulsory bytes of one MLFMA product.

    - Near-field values, nnz x (8 + index bytes).
    - Radiation and receive patterns: 2 x N x K_f x comps complex64.
    - Level patterns (boxes_l x K_l x comps complex64) moved in 4 passes:
      aggregated out, read by the translation, read by the anterpolation,
      read by the disaggregation.
    - Translation tables: 343 offsets x K_l complex64 per level.
    - x and y.

    level_boxes[l] counts the boxes of level l (0 = root); poles lists L for
    levels 2..finest, and a level samples K = 2 L^2 directions.
    comps = 3 is Cartesian level patterns (the reference's layout); comps = 2
    with near_index_bytes = 4 is the 2-component theta/phi byte model.
    radrec_comps (default: comps) counts the radiation / receive patterns
    apart: this build stores them as 2 components (theta, phi) and the level
    patterns as 3.
    """
    rr = comps if radrec_comps is None else radrec_comps
    ks = [2 * p * p for p in poles]
    boxes = list(level_boxes)[2:]
    kf = ks[-1]
    near = nnz * (8.0 + near_index_bytes)
    radrec = 2.0 * n * kf * rr * 8
    levels = sum(b * k * comps * 8.0 for b, k in zip(boxes, ks)) * 4
    trans = sum(343.0 * k * 8 for k in ks)
    return near + radrec + levels + trans + 2.0 * n * 8
