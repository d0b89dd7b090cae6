"""Volume split geometry (the reference's `cube split`): counts, offsets,
trimmed edge cubelets and output order, checked against a step-by-step
restatement of the reference's frame loop (cubelet_convert.cc:424-562)."""
import pytest

from wavelets_gb300.split import axis_count, split_grid


def reference_z_slabs(nz, size, overlap):
    """The frame loop of cube_split_typed: frames are appended until a slab
    is full, the slab is written, the next slab starts `overlap` frames back;
    leftover frames form a last, shorter slab."""
    slabs, depth, start, frame = [], 0, 0, 0
    while frame < nz:
        depth += 1
        if depth == size:
            slabs.append((start, depth))
            start = frame + 1 - overlap
            depth = 0
            if frame < nz - 1:
                frame -= overlap
        frame += 1
    if depth > 0:
        slabs.append((start, depth))
    return slabs


@pytest.mark.parametrize("n,size,overlap", [(1024, 128, 8), (248, 128, 8), (130, 128, 8),
                                            (128, 128, 8), (100, 128, 8), (77, 16, 3),
                                            (64, 16, 0), (17, 4, 1)])
def test_axis_matches_reference_frame_loop(n, size, overlap):
    slabs = reference_z_slabs(n, size, overlap)
    assert axis_count(n, size, overlap) == len(slabs)
    grid = split_grid((n, size, n), (size, size, size), overlap)
    zs = sorted({(o[2], s[2]) for o, s in grid})
    assert zs == slabs
    xs = sorted({(o[0], s[0]) for o, s in grid})
    assert xs == slabs  # x and y follow the same rule as z


def test_config_1024_cube_128_overlap_8():
    grid = split_grid((1024, 1024, 1024), (128, 128, 128), 8)
    assert len(grid) == 729
    assert grid[0] == ((0, 0, 0), (128, 128, 128))
    assert grid[8] == ((960, 0, 0), (64, 128, 128))      # edge cubelets 64 wide
    assert grid[9] == ((0, 120, 0), (128, 128, 128))     # x fastest, then y, then z
    assert grid[81] == ((0, 0, 120), (128, 128, 128))
    covered = [0] * 1024
    for (o, s) in grid[:9]:
        for x in range(o[0], o[0] + s[0]):
            covered[x] += 1
    assert min(covered) == 1 and max(covered) == 2
