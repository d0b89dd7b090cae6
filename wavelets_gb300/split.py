"""Splitting one large volume into overlapping cubelets, as the reference's
`cube split` does (cube_split_typed, cubelet_convert.cc:424-562): cubelets of
`cube` voxels that overlap their neighbours by `overlap` voxels on every
axis, the last one on an axis trimmed to the volume's end, written slab by
slab along z, rows of cubelets along y, cubelets along x.

The cubelets are not copied out: each is described by an offset into the
volume and passed to the batched compressor with the volume's row and slice
pitches."""
from typing import List, Sequence, Tuple


def axis_count(n: int, size: int, overlap: int) -> int:
    """Cubelets along one axis (cubelet_convert.cc:453-455)."""
    return (n - overlap - 1) // (size - overlap) + 1


def split_grid(volume_xyz: Sequence[int], cube_xyz: Sequence[int],
               overlap: int) -> List[Tuple[Tuple[int, int, int], Tuple[int, int, int]]]:
    """(offset, size) of every cubelet, x y z order, in the reference's output
    order."""
    counts = [axis_count(n, s, overlap) for n, s in zip(volume_xyz, cube_xyz)]
    out = []
    for kz in range(counts[2]):
        for ky in range(counts[1]):
            for kx in range(counts[0]):
                off, size = [], []
                for k, n, s in zip((kx, ky, kz), volume_xyz, cube_xyz):
                    o = k * (s - overlap)
                    off.append(o)
                    size.append(min(s, n - o))  # trimmed at the end (:475-482)
                out.append((tuple(off), tuple(size)))
    return out
