"""Host-side mesh geometry: the uniform GlobalMesh -> GlobalGrid -> LocalGrid ->
LocalMesh chain of Cabana::Grid for one rank, reduced to the scalars the
interpolation kernels consume.

Reference behaviour followed here:
  * GlobalMesh (uniform): grid/src/Cabana_Grid_GlobalMesh.hpp:47-180
    (cell count = rint(extent / cell_size), divisibility check)
  * GlobalGrid on one rank: global offset 0, owned cells = global cells,
    periodic flags (grid/src/Cabana_Grid_GlobalGrid_impl.hpp)
  * LocalGrid index spaces: grid/src/Cabana_Grid_LocalGrid_impl.hpp:49-60,
    :239-270, :430-466 (ghosted node extent = cells + 2*halo + 1)
  * LocalMesh<UniformMesh>: grid/src/Cabana_Grid_LocalMesh.hpp:61-120
    (ghost low corner = own low corner - halo * cell_size)

A mesh is 3D or 2D (UniformMesh<double, 3> / <double, 2>): the number of
entries of the corners passed to createUniformGlobalMesh sets it, and every
per-dimension tuple below has that many entries.

Pure Python; no GPU and no compiled code is needed to use it.
"""
import math
import sys
from dataclasses import dataclass, field
from typing import Sequence, Tuple

NODE = 0
CELL = 1

_EPS = sys.float_info.epsilon


class Node:
    """Entity tag (Cabana::Grid::Node)."""
    value = NODE


class Cell:
    """Entity tag (Cabana::Grid::Cell)."""
    value = CELL


@dataclass
class GlobalMesh:
    low_corner: Tuple[float, ...]
    high_corner: Tuple[float, ...]
    cell_size: Tuple[float, ...]

    @property
    def num_space_dim(self):
        return len(self.low_corner)

    def extent(self, d):
        return self.high_corner[d] - self.low_corner[d]

    def globalNumCell(self, d):
        # std::rint(extent / cell_size), GlobalMesh.hpp:155-158
        return int(round_half_even(self.extent(d) / self.cell_size[d]))

    def cellSize(self, d):
        return self.cell_size[d]

    def lowCorner(self, d):
        return self.low_corner[d]

    def highCorner(self, d):
        return self.high_corner[d]


def round_half_even(x):
    """std::rint under the default rounding mode."""
    return float(round(x))


def createUniformGlobalMesh(low_corner: Sequence[float], high_corner: Sequence[float], cell_size) -> GlobalMesh:
    """createUniformGlobalMesh for a scalar, per-dimension or cell-count argument.

    Mirrors the three GlobalMesh constructors (GlobalMesh.hpp:57-119): a scalar
    or per-dimension sequence of floats is a cell size; a sequence of ints is
    a cell count. Corners with 2 entries make a 2D mesh. Raises ValueError
    where the reference throws std::logic_error.
    """
    low = tuple(float(v) for v in low_corner)
    high = tuple(float(v) for v in high_corner)
    nd = len(low)
    if nd not in (2, 3) or len(high) != nd:
        raise ValueError("corners must both have 2 or 3 entries")
    if isinstance(cell_size, (int, float)) and not isinstance(cell_size, bool):
        cs = (float(cell_size),) * nd
        counts = None
    else:
        vals = list(cell_size)
        if all(isinstance(v, int) for v in vals):
            counts = tuple(vals)
            cs = tuple((high[d] - low[d]) / counts[d] for d in range(nd))
        else:
            counts = None
            cs = tuple(float(v) for v in vals)
    mesh = GlobalMesh(low, high, cs)
    for d in range(nd):
        ext = mesh.globalNumCell(d) * cs[d]
        if abs(ext - mesh.extent(d)) > 100.0 * _EPS:
            raise ValueError("Cabana::Grid::GlobalMesh: Extent not evenly divisible by uniform cell size")
        if counts is not None and mesh.globalNumCell(d) != counts[d]:
            raise ValueError("Cabana::Grid::GlobalMesh: Global number of cells mismatch")
    return mesh


@dataclass
class GlobalGrid:
    """One-rank GlobalGrid: the rank owns every cell (DimBlockPartitioner with a
    single block per dimension)."""
    global_mesh: GlobalMesh
    periodic: Tuple[bool, ...]

    @property
    def num_space_dim(self):
        return self.global_mesh.num_space_dim

    def globalMesh(self):
        return self.global_mesh

    def isPeriodic(self, d):
        return bool(self.periodic[d])

    def ownedNumCell(self, d):
        return self.global_mesh.globalNumCell(d)

    def globalOffset(self, d):
        return 0


def createGlobalGrid(global_mesh: GlobalMesh, is_dim_periodic=None, partitioner=None, comm=None):
    nd = global_mesh.num_space_dim
    if is_dim_periodic is None:
        is_dim_periodic = (False,) * nd
    if len(is_dim_periodic) != nd:
        raise ValueError("one periodic flag per dimension")
    return GlobalGrid(global_mesh, tuple(bool(p) for p in is_dim_periodic))


@dataclass
class LocalGrid:
    global_grid: GlobalGrid
    halo_cell_width: int

    @property
    def num_space_dim(self):
        return self.global_grid.num_space_dim

    def globalGrid(self):
        return self.global_grid

    def haloCellWidth(self):
        return self.halo_cell_width

    def totalNumCell(self, d):
        return self.global_grid.ownedNumCell(d) + 2 * self.halo_cell_width

    def ghostedExtents(self, entity=NODE):
        """Extents of indexSpace(Ghost(), entity, Local())."""
        extra = 1 if entity == NODE else 0
        return tuple(self.totalNumCell(d) + extra for d in range(self.num_space_dim))

    def ownedSpace(self, entity=NODE):
        """[min, max) per dimension of indexSpace(Own(), entity, Local())
        (LocalGrid_impl.hpp:239-250, :430-450)."""
        out = []
        hw = self.halo_cell_width
        for d in range(self.num_space_dim):
            nc = self.global_grid.ownedNumCell(d)
            if entity == NODE and not self.global_grid.isPeriodic(d):
                out.append((hw, hw + nc + 1))
            else:
                out.append((hw, hw + nc))
        return tuple(out)


def createLocalGrid(global_grid: GlobalGrid, halo_cell_width: int) -> LocalGrid:
    return LocalGrid(global_grid, int(halo_cell_width))


@dataclass
class LocalMesh:
    """LocalMesh<UniformMesh> on one rank (LocalMesh.hpp:61-120)."""
    local_grid: LocalGrid
    cell_size: Tuple[float, ...] = field(init=False)
    own_low: Tuple[float, ...] = field(init=False)
    ghost_low: Tuple[float, ...] = field(init=False)

    def __post_init__(self):
        gg = self.local_grid.global_grid
        gm = gg.global_mesh
        nd = gm.num_space_dim
        self.cell_size = tuple(gm.cellSize(d) for d in range(nd))
        self.own_low = tuple(gm.lowCorner(d) + self.cell_size[d] * gg.globalOffset(d) for d in range(nd))
        hw = self.local_grid.halo_cell_width
        self.ghost_low = tuple(self.own_low[d] - hw * self.cell_size[d] for d in range(nd))

    def coordinates(self, entity, index):
        """coordinates(Node/Cell, index) (LocalMesh.hpp:180-200)."""
        nd = len(self.cell_size)
        if entity == CELL:
            return tuple(self.ghost_low[d] + (float(index[d]) + 0.5) * self.cell_size[d] for d in range(nd))
        return tuple(self.ghost_low[d] + float(index[d]) * self.cell_size[d] for d in range(nd))


def createLocalMesh(local_grid: LocalGrid) -> LocalMesh:
    return LocalMesh(local_grid)


@dataclass(frozen=True)
class MeshParams:
    """The scalars the kernels need; field for field the cgx_mesh struct
    (per-dimension tuples have num_space_dim entries)."""
    ghost_low: Tuple[float, ...]
    cell_size: Tuple[float, ...]
    owned_cells: Tuple[int, ...]
    halo_width: int
    periodic: Tuple[int, ...]
    entity: int
    num_space_dim: int = 3

    def extents(self):
        extra = 1 if self.entity == NODE else 0
        return tuple(self.owned_cells[d] + 2 * self.halo_width + extra for d in range(self.num_space_dim))


def mesh_params(local_grid: LocalGrid, entity=NODE) -> MeshParams:
    lm = LocalMesh(local_grid)
    gg = local_grid.global_grid
    nd = local_grid.num_space_dim
    return MeshParams(
        ghost_low=lm.ghost_low,
        cell_size=lm.cell_size,
        owned_cells=tuple(gg.ownedNumCell(d) for d in range(nd)),
        halo_width=local_grid.halo_cell_width,
        periodic=tuple(int(gg.isPeriodic(d)) for d in range(nd)),
        entity=int(entity),
        num_space_dim=nd,
    )


def simple_mesh(cells, cell_size=1.0, low=(0.0, 0.0, 0.0), halo_width=1, periodic=(False, False, False), entity=NODE):
    """Convenience: a cubic-cell mesh of `cells` owned cells starting at `low`."""
    if isinstance(cells, int):
        cells = (cells,) * 3
    high = tuple(low[d] + cells[d] * cell_size for d in range(3))
    gm = createUniformGlobalMesh(low, high, cell_size)
    lg = createLocalGrid(createGlobalGrid(gm, periodic), halo_width)
    return lg, mesh_params(lg, entity)


def cartesian_num_bins(grid_min, grid_max, grid_delta):
    """CartesianGrid::init cell counts (core/src/impl/Cabana_CartesianGrid.hpp:61-73)."""
    return tuple(int(math.floor((grid_max[d] - grid_min[d]) * (1.0 / grid_delta[d]))) for d in range(3))
