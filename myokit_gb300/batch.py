"""
Batched tissues: many independent cables or sheets of uneven size and
parameter sets in one :class:`SimulationCUDA`, so that they advance in one
persistent launch (one grid barrier per step for all of them) instead of one
launch stream per tissue.

The reference expresses the same thing with one 1D ``SimulationOpenCL``
whose ``set_connections`` chains stop at cable boundaries, a
``set_paced_cell_list`` and per-cell ``set_field`` values
(``openclsim.py:1387-1449, 1534-1629``). Here cables become one 1D
heterogeneous-conductance simulation with zero conductance between cables
(neighbour reads stay on the regular, staged fast path), and sheets are
packed side by side in one 2D heterogeneous grid whose conductances are
zero across sheet borders and around the padding below shorter sheets.
"""
import numpy as np

from ._deps import myokit
from .simulation import SimulationCUDA


class CableBatch(object):
    """
    ``len(lengths)`` independent cables in one simulation.

    ``lengths``
        Cells per cable.
    ``conductance``
        Conductance between neighbouring cells of a cable (scalar, or one
        value per cable).
    ``paced_cells``
        The first ``paced_cells`` cells of every cable are paced.
    ``fields``
        ``{variable: values}``: one value per cable (broadcast to its cells)
        or one per cell of the batch.

    Other keyword arguments go to :class:`SimulationCUDA`. Cable ``c``
    holds cells ``starts[c]`` to ``starts[c] + lengths[c] - 1``; ``sim`` is
    the simulation, used like any other.
    """
    def __init__(self, model, lengths, protocol=None, conductance=9.0,
                 paced_cells=5, fields=None, **kwargs):
        self.lengths = np.asarray(lengths, dtype=np.int64)
        if self.lengths.ndim != 1 or len(self.lengths) < 1:
            raise ValueError('lengths must be a non-empty 1d sequence')
        if np.any(self.lengths < 1):
            raise ValueError('Every cable needs at least one cell.')
        self.starts = np.concatenate(
            [[0], np.cumsum(self.lengths)[:-1]]).astype(np.int64)
        self.ncells = int(self.lengths.sum())
        self.sim = SimulationCUDA(model, protocol, ncells=self.ncells,
                                  **kwargs)
        if self.ncells > 1:
            self.sim.set_conductance_field(self.edge_conductances(
                conductance))
        paced = self.paced_cells(paced_cells)
        if len(paced):
            self.sim.set_paced_cell_list(paced)
        for name, values in (fields or {}).items():
            self.sim.set_field(name, self.per_cell(values))

    def edge_conductances(self, conductance):
        """Conductances of the ncells - 1 edges: g inside, 0 between."""
        g = np.broadcast_to(np.asarray(conductance, dtype=float),
                            (len(self.lengths),))
        edges = np.repeat(g, self.lengths)[:-1].copy()
        edges[self.starts[1:] - 1] = 0
        return edges

    def paced_cells(self, n):
        """Cell ids of the first ``n`` cells of every cable."""
        n = int(n)
        return [int(a + k) for a, ln in zip(self.starts, self.lengths)
                for k in range(min(n, int(ln)))]

    def per_cell(self, values):
        """Per-cable values broadcast to cells (per-cell values pass)."""
        v = np.asarray(values, dtype=float)
        if v.shape == (len(self.lengths),):
            return np.repeat(v, self.lengths)
        if v.shape == (self.ncells,):
            return v
        raise ValueError('Field values must have one entry per cable or'
                         ' per cell.')

    def cable_state(self, c, state=None):
        """State of cable ``c``, shaped (cells, states)."""
        st = self.sim.state_array() if state is None else np.asarray(state)
        st = st.reshape(self.ncells, -1)
        a = int(self.starts[c])
        return st[a:a + int(self.lengths[c])]

    def cable_log_keys(self, c, variable='membrane.V'):
        """Log keys of one variable over the cells of cable ``c``."""
        a = int(self.starts[c])
        return ['%d.%s' % (a + k, variable)
                for k in range(int(self.lengths[c]))]


class SheetBatch(object):
    """
    Independent sheets of uneven size in one 2D simulation. Sheets are placed
    side by side (sheet ``i`` starts at column ``x0[i]``) in a grid as high
    as the tallest sheet; cells below a shorter sheet are padding: they are
    computed but unpaced and connected to nothing.

    ``shapes``
        ``(nx, ny)`` of each sheet.
    ``conductance``
        ``(gx, gy)`` inside every sheet, or one pair per sheet.
    ``paced_columns``
        The first ``paced_columns`` columns of every sheet are paced.
    ``fields``
        ``{variable: values}``: one value per sheet, or one array per sheet
        shaped ``(ny, nx)`` of that sheet.
    """
    def __init__(self, model, shapes, protocol=None, conductance=(9.0, 9.0),
                 paced_columns=4, fields=None, **kwargs):
        self.shapes = [(int(a), int(b)) for a, b in shapes]
        if not self.shapes or min(min(s) for s in self.shapes) < 1:
            raise ValueError('Every sheet needs at least one cell.')
        widths = np.array([s[0] for s in self.shapes])
        self.x0 = np.concatenate([[0], np.cumsum(widths)[:-1]]).astype(int)
        self.nx = int(widths.sum())
        self.ny = max(s[1] for s in self.shapes)
        self.sim = SimulationCUDA(model, protocol, ncells=(self.nx, self.ny),
                                  **kwargs)
        gx, gy = self.edge_conductances(conductance)
        self.sim.set_conductance_field(gx, gy)
        paced = self.paced_cells(paced_columns)
        if paced:
            self.sim.set_paced_cell_list(paced)
        for name, values in (fields or {}).items():
            var = name if isinstance(name, myokit.Variable) else \
                model.get(name)
            self.sim.set_field(name, self.per_cell(values, var.eval()))

    def _pairs(self, conductance):
        c = np.asarray(conductance, dtype=float)
        if c.shape == (2,):
            return [tuple(c)] * len(self.shapes)
        if c.shape == (len(self.shapes), 2):
            return [tuple(x) for x in c]
        raise ValueError('conductance must be (gx, gy) or one pair per'
                         ' sheet')

    def edge_conductances(self, conductance):
        """Per-edge gx (ny, nx - 1) and gy (ny - 1, nx) of the packed grid."""
        gx = np.zeros((self.ny, max(self.nx - 1, 0)))
        gy = np.zeros((max(self.ny - 1, 0), self.nx))
        for (w, h), x0, (cx, cy) in zip(self.shapes, self.x0,
                                        self._pairs(conductance)):
            if w > 1:
                gx[:h, x0:x0 + w - 1] = cx
            if h > 1:
                gy[:h - 1, x0:x0 + w] = cy
        return gx, gy

    def paced_cells(self, ncols):
        """(x, y) of the cells in the first ``ncols`` columns of every
        sheet."""
        out = []
        for (w, h), x0 in zip(self.shapes, self.x0):
            for y in range(h):
                for x in range(min(int(ncols), w)):
                    out.append((int(x0 + x), y))
        return out

    def per_cell(self, values, pad=0.0):
        """Per-sheet scalars or per-sheet arrays on the packed grid;
        padding cells get ``pad`` (the variable's own value)."""
        grid = np.full((self.ny, self.nx), float(pad))
        if np.ndim(values) == 1 and len(values) == len(self.shapes):
            values = [np.full((h, w), float(v))
                      for v, (w, h) in zip(values, self.shapes)]
        if len(values) != len(self.shapes):
            raise ValueError('Field values must have one entry per sheet.')
        for v, (w, h), x0 in zip(values, self.shapes, self.x0):
            v = np.asarray(v, dtype=float)
            if v.shape != (h, w):
                raise ValueError('A sheet field must be shaped (ny, nx).')
            grid[:h, x0:x0 + w] = v
        return grid

    def sheet_state(self, i, state=None):
        """State of sheet ``i``, shaped (ny, nx, states)."""
        st = self.sim.state_array() if state is None else np.asarray(state)
        st = st.reshape(self.ny, self.nx, -1)
        w, h = self.shapes[i]
        x0 = int(self.x0[i])
        return st[:h, x0:x0 + w]

    def sheet_frames(self, i, frames):
        """Sheet ``i`` cut out of frames shaped (n, ny, nx)."""
        w, h = self.shapes[i]
        x0 = int(self.x0[i])
        return frames[:, :h, x0:x0 + w]


def frames_to_block(times, frames, name='membrane.V'):
    """
    A ``myokit.DataBlock2d`` holding device frames (as returned by
    :meth:`SimulationCUDA.run_frames`) of a 2D simulation, for the reference's
    block tools (``DataBlock2d.save``, ``images``, ...); copies to the host.
    """
    data = frames.detach().cpu().double().numpy() if hasattr(
        frames, 'detach') else np.asarray(frames, dtype=float)
    if data.ndim != 3:
        raise ValueError('Frames of a 2D simulation are shaped (n, ny, nx).')
    n, ny, nx = data.shape
    block = myokit.DataBlock2d(nx, ny, np.asarray(times, dtype=float))
    block.set2d(name, data)
    return block
