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


_README_FRAMES = (
    'Frames recorded on the device by myokit_gb300, in the file format of\n'
    'myokit.DataBlock{d}d.save: header_block{d}d.txt holds nt, {dims}the\n'
    'data type and the entry names; data.bin holds little-endian doubles:\n'
    'the nt times, then each {d}d entry in C order.\n')


def save_frames(path, times, frames, name='membrane.V', chunk=16):
    """
    Writes device frames (as returned by :meth:`SimulationCUDA.run_frames`)
    to ``path`` in the file format of ``myokit.DataBlock2d.save`` (frames
    shaped ``(n, ny, nx)``) or ``myokit.DataBlock1d.save`` (``(n, nx)``),
    ``myokit/_datablock.py:1423-1500, 631-704``: a zip archive holding a
    text header, ``data.bin`` (little-endian doubles: the times, then every
    entry in C order) and a readme. The frames are copied to the host
    ``chunk`` at a time and streamed into the archive, so the host never
    holds the whole block; ``myokit.DataBlock2d.load`` (or ``1d``) reads the
    file. ``frames`` is one tensor or array, stored as ``name``, or a dict
    ``{name: frames}`` of equally shaped frame sets.
    """
    import os
    import zipfile
    sets = dict(frames) if isinstance(frames, dict) else {name: frames}
    if not sets:
        raise ValueError('No frames to save.')
    t = np.ascontiguousarray(times, dtype='<f8')
    shape = None
    for k, f in sets.items():
        s = tuple(f.shape)
        if len(s) not in (2, 3):
            raise ValueError('Frames are shaped (n, nx) or (n, ny, nx).')
        if shape is not None and s != shape:
            raise ValueError('Every frame set must have the same shape.')
        shape = s
    if shape[0] != len(t):
        raise ValueError('One time per frame is needed.')
    chunk = max(1, int(chunk))
    d = len(shape) - 1
    head = [str(shape[0])] + [str(x) for x in shape[1:]] + ['"d"', str(d)]
    head += ['"%s"' % k for k in sets]

    def host(f, i, j):
        # Frames i..j-1 as host doubles (torch tensors on any device, or
        # arrays)
        if hasattr(f, 'detach'):
            import torch
            return f[i:j].detach().to('cpu', torch.float64).numpy()
        return np.asarray(f[i:j], dtype=np.float64)

    with zipfile.ZipFile(os.path.expanduser(path), 'w',
                         compression=zipfile.ZIP_DEFLATED,
                         allowZip64=True) as z:
        z.writestr('header_block%dd.txt' % d, '\n'.join(head))
        with z.open('data.bin', 'w', force_zip64=True) as out:
            out.write(t.tobytes())
            for f in sets.values():
                for i in range(0, shape[0], chunk):
                    block = host(f, i, min(shape[0], i + chunk))
                    out.write(np.ascontiguousarray(block, '<f8').tobytes())
        dims = 'ny, nx, ' if d == 2 else 'nx, '
        z.writestr('readme.txt', _README_FRAMES.format(d=d, dims=dims))
