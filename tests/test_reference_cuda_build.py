"""The reference's kernels built for the GPU (oracle/ref/build.py build_gpu; run on the GPU by oracle/ref_cuda.py):
the cubins and the argument layout exist where the reference checkout is present, the layout is the one the
launcher packs (field offsets inside their structs, sizes of the by-value arguments), and kernel names are read
from mangled names as the launcher reads them. No GPU is used here."""
import json

import pytest

from oracle import ref_cuda
from oracle.ref import build as ref_build

needs_ref = pytest.mark.skipif(not ref_build.available(), reason="the reference checkout is not present")


def test_kernel_names_from_mangled_names():
    n = ref_cuda._kernel_name
    assert n("_ZN3sph4cuda6kernel16computeDensitiesENS0_18FluidParticlesDataENS0_12NeighborGrid6DeviceE") == \
        "computeDensities"
    assert n("_ZN3sph4cuda6kernel31calculateCellStartAndEndIndicesENS0_12NeighborGrid8GridDataE") == \
        "calculateCellStartAndEndIndices"
    assert n("_ZN3sph4cuda10refinement15splitParticlesE") is None


@needs_ref
def test_cubins_and_layout_built():
    outs = ref_build.build_gpu()
    assert len(outs) == len(ref_build.GPU_SOURCES) + 1
    with open(ref_build.LAYOUT) as f:
        L = json.load(f)
    # pointers are 8 bytes, counts 4; the structs as the launcher packs them
    F = L["FluidParticlesData"]
    assert [F[k] for k in ("positions", "velocities", "accelerations", "densities", "radii", "smoothingRadii",
                           "masses", "particleCount")] == [0, 8, 16, 24, 32, 40, 48, 56] and F["size"] == 64
    G = L["GridData"]
    assert G["particleCount"] == 64 and G["size"] == 72
    for k in ("cellStartIndices", "cellEndIndices", "particleGridIndices", "particleArrayIndices"):
        assert G[k + ".size"] == G[k + ".data"] + 8
    D = L["Device"]
    assert D["grid"] >= L["Domain"]["size"] and D["fluid"] % 8 == 0 and D["boundary"] == D["fluid"] + G["size"]
    P = L["Parameters"]
    assert P["threadsPerBlock"] + 4 == P["size"] and L["wendlandRangeRatio"] == 2.0
    for kernel, (module, kinds) in ref_cuda.KERNELS.items():
        assert module in ref_cuda.MODULES and kinds
