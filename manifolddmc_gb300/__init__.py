"""manifolddmc_gb300: Dual Marching Cubes with non-manifold repair on GB300.

Python mirror of the reference's DMC interface (PhiliGuertler/ManifoldDMC,
MarchingCubes/VisualDMC/src/DMC/DualMarchingCubes.h, UniformGrid.h) over the
C ABI of the in-tree CUDA library (include/mdmc.h).  Names follow the
reference in snake_case: ``DualMarchingCubes.run(iso_value, grid)``,
``get_num_non_manifold_edges4()``, ``set_splitting_step(...)``,
``UniformGrid.read_from_file(path, refinement, add_zero_boundary)``.

The compute path is the CUDA library only; when it cannot be loaded every
entry point raises ``RuntimeError`` (there is no CPU fallback).
"""
import ctypes
import threading
from pathlib import Path

import numpy as np

from .build import LIB as _LIB_PATH
from .build import build

__all__ = ["DualMarchingCubes", "UniformGrid", "HalfedgeMesh", "SplittingStep", "Options", "Stats",
           "library", "build", "MDMCError"]

# SplittingStep, PostProcesses/ManifoldSplitter.h:155-166
class SplittingStep:
    NONE = 0
    SUBDIVIDE_QUADS = 1
    COLLAPSE_NON_MANIFOLD_EDGES = 2
    MERGE_VERTICES = 3
    UPDATE_HALFEDGE_TWINS = 4
    MOVE_VERTICES_TO_SURFACE = 5
    ENABLE_ITERATIVE_REFINEMENT = 6
    ALL = 100


class Options(ctypes.Structure):
    _fields_ = [("enable_surface_to_vertex_iteration", ctypes.c_int),
                ("simplify_p3x3y_color", ctypes.c_int),
                ("simplify_p3x3y_old", ctypes.c_int),
                ("simplify_p3333", ctypes.c_int),
                ("split_non_manifold_halfedges", ctypes.c_int),
                ("detect_non_manifold_vertices", ctypes.c_int),
                ("splitting_step", ctypes.c_int)]


class Grid(ctypes.Structure):
    _fields_ = [("samples", ctypes.c_void_p),
                ("dims", ctypes.c_int32 * 3),
                ("origin", ctypes.c_float * 3),
                ("spacing", ctypes.c_float * 3),
                ("coarse_samples", ctypes.c_void_p),
                ("coarse_dims", ctypes.c_int32 * 3),
                ("refinement", ctypes.c_int32),
                ("add_zero_boundary", ctypes.c_int32)]


class Mesh(ctypes.Structure):
    _fields_ = [("num_vertices", ctypes.c_int64), ("num_faces", ctypes.c_int64),
                ("num_halfedges", ctypes.c_int64),
                ("positions", ctypes.c_void_p), ("normals", ctypes.c_void_p), ("quads", ctypes.c_void_p),
                ("halfedges", ctypes.c_void_p), ("face_first_halfedge", ctypes.c_void_p),
                ("face_attributes", ctypes.c_void_p), ("vertex_halfedge", ctypes.c_void_p),
                ("vertex_flags", ctypes.c_void_p)]


class HostMeshArrays(ctypes.Structure):
    _fields_ = [("capacity_vertices", ctypes.c_int64), ("capacity_faces", ctypes.c_int64),
                ("positions", ctypes.c_void_p), ("normals", ctypes.c_void_p), ("quads", ctypes.c_void_p),
                ("halfedges", ctypes.c_void_p), ("face_first_halfedge", ctypes.c_void_p),
                ("face_attributes", ctypes.c_void_p), ("vertex_halfedge", ctypes.c_void_p),
                ("vertex_flags", ctypes.c_void_p)]


class HostMesh:
    """Page-locked host arrays for DualMarchingCubes.run_to_host, for meshes
    of up to max_vertices vertices and max_faces faces."""

    def __init__(self, max_vertices, max_faces):
        import torch
        V, F = int(max_vertices), int(max_faces)

        def pinned(shape, dtype):
            return torch.empty(shape, dtype=dtype).pin_memory()

        self.tensors = {"positions": pinned((V, 3), torch.float32), "normals": pinned((V, 3), torch.float32),
                        "quads": pinned((F, 4), torch.int32), "halfedges": pinned((4 * F, 4), torch.int32),
                        "face_first_halfedge": pinned((F,), torch.int32),
                        "face_attributes": pinned((F,), torch.int16),
                        "vertex_halfedge": pinned((V,), torch.int32), "vertex_flags": pinned((V,), torch.uint8)}
        self.arrays = HostMeshArrays(V, F, *[t.data_ptr() for t in self.tensors.values()])

    def mesh(self, V, F):
        """numpy views of the first V vertices and F faces"""
        t = self.tensors
        return HalfedgeMesh(t["positions"][:V].numpy(), t["normals"][:V].numpy(), t["quads"][:F].numpy(),
                            t["halfedges"][:4 * F].numpy(), t["face_first_halfedge"][:F].numpy(),
                            t["face_attributes"][:F].numpy().view(np.uint16), t["vertex_halfedge"][:V].numpy(),
                            t["vertex_flags"][:V].numpy())


class TriangleMesh(ctypes.Structure):
    _fields_ = [("num_vertices", ctypes.c_int64), ("num_triangles", ctypes.c_int64),
                ("positions", ctypes.c_void_p), ("normals", ctypes.c_void_p), ("triangles", ctypes.c_void_p)]


class Stats(ctypes.Structure):
    _fields_ = [("num_dmc_vertices", ctypes.c_int64), ("num_dmc_quads", ctypes.c_int64),
                ("num_active_cells", ctypes.c_int64), ("num_edges", ctypes.c_int64),
                ("num_edges3", ctypes.c_int64), ("num_edges4", ctypes.c_int64),
                ("num_non_manifold_vertices", ctypes.c_int64),
                ("quads_with_non_manifold_edges", ctypes.c_int64 * 4),
                ("split_iterations", ctypes.c_int64), ("anomalies", ctypes.c_int64),
                ("ms_dmc", ctypes.c_float), ("ms_halfedge", ctypes.c_float), ("ms_repair", ctypes.c_float),
                ("ms_detect", ctypes.c_float), ("ms_total", ctypes.c_float),
                ("ms_refine", ctypes.c_float), ("ms_count", ctypes.c_float), ("ms_emit", ctypes.c_float),
                ("ms_vertices", ctypes.c_float),
                ("ms_quads", ctypes.c_float), ("ms_table", ctypes.c_float), ("kernel_launches", ctypes.c_int64)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "quads_with_non_manifold_edges"}
        d["quads_with_non_manifold_edges"] = list(self.quads_with_non_manifold_edges)
        return d


STATUS = {0: "ok", 1: "invalid argument", 2: "cuda error", 3: "out of memory", 4: "device limit hit",
          5: "io error", 6: "no cuda device"}

# kernels mdmc_set_kernel_timing can time (MDMC_TIME_* of mdmc.h) -> Stats field
KERNEL_TIMING = {"refine": (1, "ms_refine"), "count": (2, "ms_count"), "emit": (4, "ms_emit"),
                 "quads": (8, "ms_quads"), "table": (16, "ms_table"), "vertices": (32, "ms_vertices")}
TIME_STAGES = 64  # the stage times (on by default)
TIME_ALL = 127


class MDMCError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (%d): %s" % (STATUS.get(status, "error"), status, message))
        self.status = status


_lock = threading.Lock()
_lib = None
P = ctypes.c_void_p


def library():
    """Loads libmdmc.so (building it when missing).  Raises when it cannot."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not _LIB_PATH.exists():
            build()
        if not _LIB_PATH.exists():
            raise RuntimeError("libmdmc.so is missing; run manifolddmc_gb300.build.build()")
        lib = ctypes.CDLL(str(_LIB_PATH))
        sig = {
            "mdmc_default_options": (None, [P]),
            "mdmc_create": (ctypes.c_int, [P, P]),
            "mdmc_destroy": (None, [P]),
            "mdmc_set_options": (ctypes.c_int, [P, P]),
            "mdmc_set_kernel_timing": (ctypes.c_int, [P, ctypes.c_uint32]),
            "mdmc_get_options": (ctypes.c_int, [P, P]),
            "mdmc_read_bin": (ctypes.c_int, [ctypes.c_char_p, P, P, P, P]),
            "mdmc_prepare_grid": (ctypes.c_int, [P, P, ctypes.c_int, P, P, P, ctypes.c_int32, ctypes.c_int32, P, P]),
            "mdmc_run": (ctypes.c_int, [P, P, ctypes.c_float, P, P, P]),
            "mdmc_materialize_grid": (ctypes.c_int, [P, P, P, P]),
            "mdmc_get_mesh": (ctypes.c_int, [P, P]),
            "mdmc_get_stats": (ctypes.c_int, [P, P]),
            "mdmc_download_mesh": (ctypes.c_int, [P] * 10),
            "mdmc_write_obj": (ctypes.c_int, [P, ctypes.c_char_p]),
            "mdmc_last_error": (ctypes.c_char_p, [P]),
            "mdmc_case_tables": (None, [P, P]),
            "mdmc_backward": (ctypes.c_int, [P, P, P, ctypes.c_int, P]),
            "mdmc_render_buffers": (ctypes.c_int, [P, P, P, P]),
            "mdmc_run_standard_mc": (ctypes.c_int, [P, P, ctypes.c_float, P, P]),
            "mdmc_run_to_host": (ctypes.c_int, [P, P, ctypes.c_float, P, P, P, P]),
            "mdmc_download_triangle_mesh": (ctypes.c_int, [P] * 5),
            "mdmc_color_faces": (ctypes.c_int, [P, P]),
            "mdmc_quads_to_triangles": (ctypes.c_int, [P, ctypes.c_int64, P, P]),
            "mdmc_mean_ratio": (ctypes.c_int, [P, ctypes.c_int64, P, ctypes.c_int64, P, P, P]),
            "mdmc_generate_volume": (ctypes.c_int, [ctypes.c_int32, P, P, P, P, P]),
            "mdmc_generate_edge_case": (ctypes.c_int, [ctypes.c_int32, P, P, P, P, P]),
            "mdmc_write_bin": (ctypes.c_int, [ctypes.c_char_p, P, P, P]),
            "mdmc_batch_create": (ctypes.c_int, [P, P, ctypes.c_int]),
            "mdmc_batch_destroy": (None, [P]),
            "mdmc_run_batch": (ctypes.c_int, [P, P, P, ctypes.c_int, P, P, P]),
            "mdmc_batch_streams": (ctypes.c_int, [P]),
            "mdmc_batch_context": (P, [P, ctypes.c_int]),
            "mdmc_batch_last_error": (ctypes.c_char_p, [P]),
            "mdmc_point_index_create": (ctypes.c_int, [P, P, ctypes.c_int64, P]),
            "mdmc_point_index_destroy": (None, [P]),
            "mdmc_point_index_nearest": (ctypes.c_int, [P, P, ctypes.c_int64, P, P, P, P]),
            "mdmc_point_index_count": (ctypes.c_int64, [P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def _ptr(a):
    return a.ctypes.data_as(P) if a is not None else None


def _dev_ptr(a):
    """Device address of a CUDA tensor, an integer, or None."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return int(a)


class _DeviceArray:
    """A view of library-owned device memory for torch.as_tensor (CUDA array interface)."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr or 0), False),
                                         "version": 2, "strides": None}


def _stream_handle(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream", stream))


class _Context:
    def __init__(self, options=None):
        self.lib = library()
        self.handle = P()
        st = self.lib.mdmc_create(ctypes.byref(self.handle), ctypes.byref(options) if options is not None else None)
        if st != 0:
            raise MDMCError(st, "mdmc_create failed")

    def check(self, st):
        if st != 0:
            raise MDMCError(st, self.lib.mdmc_last_error(self.handle).decode())

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            self.lib.mdmc_destroy(h)
            self.handle = None


def read_bin(path):
    """UniformGridHost::readFromFile<unsigned short> (UniformGrid.inl:512-571) on the host.
    Returns (samples float32 [z,y,x], dims, spacing, origin)."""
    lib = library()
    dims = np.zeros(3, np.int32)
    sp = np.zeros(3, np.float32)
    org = np.zeros(3, np.float32)
    st = lib.mdmc_read_bin(str(path).encode(), _ptr(dims), _ptr(sp), _ptr(org), None)
    if st != 0:
        raise MDMCError(st, "cannot read %s" % path)
    out = np.empty(int(np.prod(dims)), np.float32)
    lib.mdmc_read_bin(str(path).encode(), _ptr(dims), _ptr(sp), _ptr(org), _ptr(out))
    return out.reshape(dims[2], dims[1], dims[0]), [int(d) for d in dims], sp, org


class UniformGrid:
    """A uniform float grid on the device (UniformGridHost<float>, UniformGrid.h:264-430).

    ``samples`` may be a numpy array (host, copied in) or a CUDA torch tensor
    / integer device pointer (used in place when no refinement or padding is
    asked for)."""

    def __init__(self, samples, dims=None, origin=(0.0, 0.0, 0.0), spacing=(1.0, 1.0, 1.0), refinement=0,
                 add_zero_boundary=False, stream=None):
        self._ctx = _Context()
        self._keep = samples
        if isinstance(samples, np.ndarray):
            arr = np.ascontiguousarray(samples, np.float32)
            if dims is None:
                dims = [arr.shape[2], arr.shape[1], arr.shape[0]]
            self._keep = arr
            ptr, on_host = arr.ctypes.data, 1
        elif hasattr(samples, "data_ptr"):
            if dims is None:
                dims = [samples.shape[2], samples.shape[1], samples.shape[0]]
            ptr, on_host = samples.data_ptr(), 0
        else:
            ptr, on_host = int(samples), 0
        d = np.asarray(dims, np.int32)
        o = np.asarray(origin, np.float32)
        s = np.asarray(spacing, np.float32)
        self.grid = Grid()
        self._ctx.check(self._ctx.lib.mdmc_prepare_grid(self._ctx.handle, P(ptr), on_host, _ptr(d), _ptr(o), _ptr(s),
                                                        int(refinement), int(bool(add_zero_boundary)),
                                                        ctypes.byref(self.grid), _stream_handle(stream)))

    @classmethod
    def read_from_file(cls, path, refinement=0, add_zero_boundary=False):
        """UniformGridHost::readFromFile(file, refinement, addZeroBoundary), UniformGrid.inl:575-608"""
        samples, dims, sp, org = read_bin(path)
        return cls(samples, dims, org, sp, refinement, add_zero_boundary)

    @property
    def dimensions(self):
        return [int(x) for x in self.grid.dims]

    @property
    def origin(self):
        return np.array(list(self.grid.origin), np.float32)

    @property
    def deltas(self):
        return np.array(list(self.grid.spacing), np.float32)

    def get_cell_count(self):
        d = self.dimensions
        return d[0] * d[1] * d[2]

    def materialize(self, out_device_ptr, stream=None):
        """Writes the dense (refined) samples to a device buffer of get_cell_count() floats."""
        self._ctx.check(self._ctx.lib.mdmc_materialize_grid(self._ctx.handle, ctypes.byref(self.grid),
                                                            P(int(out_device_ptr)), _stream_handle(stream)))


class HalfedgeMesh:
    """Host copy of the halfedge mesh (HalfedgeMesh, Halfedges/HalfedgeMesh.h)."""

    def __init__(self, positions, normals, quads, halfedges, face_first_halfedge, face_attributes, vertex_halfedge,
                 vertex_flags):
        self.positions = positions
        self.normals = normals
        self.quads = quads
        self.halfedges = halfedges
        self.face_first_halfedge = face_first_halfedge
        self.face_attributes = face_attributes
        self.vertex_halfedge = vertex_halfedge
        self.vertex_flags = vertex_flags


class DualMarchingCubes:
    """DMC::DualMarchingCubes (DualMarchingCubes.h:68-186) on the GPU."""

    def __init__(self, **flags):
        lib = library()
        self.options = Options()
        lib.mdmc_default_options(ctypes.byref(self.options))
        for k, v in flags.items():
            setattr(self.options, k, int(v))
        self._ctx = _Context(self.options)
        self.stats = Stats()
        self.mesh = Mesh()
        self._run_id = 0

    # flags (DualMarchingCubes.h:167-185, defaults DualMarchingCubes.cu:110-133)
    def _set(self, name, value):
        setattr(self.options, name, int(value))
        self._ctx.check(self._ctx.lib.mdmc_set_options(self._ctx.handle, ctypes.byref(self.options)))

    def set_splitting_step(self, step):
        """DualMarchingCubes::setSplittingStep, DualMarchingCubes.h:143-145"""
        self._set("splitting_step", step)

    def set_option(self, name, value):
        self._set(name, value)

    def set_kernel_timing(self, kernels, stages=True):
        """Times the named kernels (keys of KERNEL_TIMING; or an MDMC_TIME_*
        mask, used as given) and, with stages, the stage times in the following
        runs' stats; every timed item costs event records on the stream."""
        if isinstance(kernels, int):
            mask = kernels
        else:
            mask = sum(KERNEL_TIMING[k][0] for k in kernels) | (TIME_STAGES if stages else 0)
        self._ctx.check(self._ctx.lib.mdmc_set_kernel_timing(self._ctx.handle, mask))

    def run(self, iso_value, grid, stream=None):
        """DualMarchingCubes::run, DualMarchingCubes.cu:220-289.  Returns the
        per-stage GPU times in milliseconds (the reference returns its
        Performance tree)."""
        g = grid.grid if isinstance(grid, UniformGrid) else grid
        self._run_id += 1
        self._ctx.check(self._ctx.lib.mdmc_run(self._ctx.handle, ctypes.byref(g), ctypes.c_float(iso_value),
                                               ctypes.byref(self.mesh), ctypes.byref(self.stats),
                                               _stream_handle(stream)))
        s = self.stats
        return {"DMC": s.ms_dmc, "HalfedgeMesh": s.ms_halfedge, "Repair": s.ms_repair,
                "DetectNonManifoldVertices": s.ms_detect, "Total": s.ms_total}

    def run_to_host(self, iso_value, grid, host, stream=None):
        """run() with the mesh copied into the HostMesh `host` while the run
        goes on (mdmc_run_to_host); returns numpy views of host's arrays
        holding the mesh."""
        g = grid.grid if isinstance(grid, UniformGrid) else grid
        self._run_id += 1
        self._ctx.check(self._ctx.lib.mdmc_run_to_host(self._ctx.handle, ctypes.byref(g), ctypes.c_float(iso_value),
                                                       ctypes.byref(host.arrays), ctypes.byref(self.mesh),
                                                       ctypes.byref(self.stats), _stream_handle(stream)))
        return host.mesh(int(self.mesh.num_vertices), int(self.mesh.num_faces))

    # statistics getters (DualMarchingCubes.h:87-118)
    def get_num_vertices(self):
        return int(self.stats.num_dmc_vertices)

    def get_num_quads(self):
        return int(self.stats.num_dmc_quads)

    def get_num_non_manifold_edges4(self):
        return int(self.stats.num_edges4)

    def get_num_non_manifold_edges3(self):
        return int(self.stats.num_edges3)

    def get_num_edges(self):
        return int(self.stats.num_edges)

    def get_num_non_manifold_vertices(self):
        return int(self.stats.num_non_manifold_vertices)

    def get_num_quads_with_non_manifold_edges(self, k):
        if not 1 <= k <= 4:
            return 0
        return int(self.stats.quads_with_non_manifold_edges[k - 1])

    def get_halfedge_mesh(self):
        """The last run's mesh copied to host numpy arrays."""
        m = self.mesh
        V, F, H = int(m.num_vertices), int(m.num_faces), int(m.num_halfedges)
        out = HalfedgeMesh(np.empty((V, 3), np.float32), np.empty((V, 3), np.float32), np.empty((F, 4), np.int32),
                           np.empty((H, 4), np.int32), np.empty(F, np.int32), np.empty(F, np.uint16),
                           np.empty(V, np.int32), np.empty(V, np.uint8))
        self._ctx.check(self._ctx.lib.mdmc_download_mesh(
            self._ctx.handle, _ptr(out.positions), _ptr(out.normals), _ptr(out.quads), _ptr(out.halfedges),
            _ptr(out.face_first_halfedge), _ptr(out.face_attributes), _ptr(out.vertex_halfedge),
            _ptr(out.vertex_flags), None))
        return out

    def device_arrays(self, names=None):
        """The last run's mesh as CUDA torch tensors viewing the library's
        buffers (valid until the next run on this object); `names` picks a
        subset (all by default)."""
        import torch
        m = self.mesh
        V, F, H = int(m.num_vertices), int(m.num_faces), int(m.num_halfedges)
        views = {"positions": (m.positions, (V, 3), "<f4"), "normals": (m.normals, (V, 3), "<f4"),
                 "quads": (m.quads, (F, 4), "<i4"), "halfedges": (m.halfedges, (H, 4), "<i4"),
                 "face_first_halfedge": (m.face_first_halfedge, (F,), "<i4"),
                 "vertex_halfedge": (m.vertex_halfedge, (V,), "<i4"), "vertex_flags": (m.vertex_flags, (V,), "|u1")}
        if names is not None:
            views = {k: views[k] for k in names}
        out = {}
        for k, (ptr, shape, ts) in views.items():
            addr = int(ptr) if ptr else 0
            if not addr or 0 in shape:
                out[k] = torch.empty(shape, dtype={"<f4": torch.float32, "<i4": torch.int32, "|u1": torch.uint8}[ts],
                                     device="cuda")
            else:
                out[k] = torch.as_tensor(_DeviceArray(addr, shape, ts), device="cuda")
        return out

    def backward(self, dl_dpositions, dl_dsamples, accumulate=False, stream=None):
        """Adjoint of the last run (no counterpart in the reference): writes
        dL/dsamples of the grid the run read (the coarse input of a refined
        grid) from dL/dpositions (3 floats per vertex), topology held fixed.
        Needs a run with enable_surface_to_vertex_iteration = 0."""
        self._ctx.check(self._ctx.lib.mdmc_backward(self._ctx.handle, _dev_ptr(dl_dpositions), _dev_ptr(dl_dsamples),
                                                    int(bool(accumulate)), _stream_handle(stream)))

    def render_buffers(self, vertices=None, indices=None, stream=None):
        """HalfedgeMesh::toVertexAndIndexBuffer (HalfedgeMesh.cu:1102-1146) into
        CUDA tensors: vertices [V, 10] float32 (position, normal, rgba) and
        indices [F * 6] uint32 (two triangles per quad).  Allocates them when
        not given."""
        import torch
        V, F = int(self.mesh.num_vertices), int(self.mesh.num_faces)
        if vertices is None:
            vertices = torch.empty((V, 10), dtype=torch.float32, device="cuda")
        if indices is None:
            indices = torch.empty(6 * F, dtype=torch.int32, device="cuda")
        self._ctx.check(self._ctx.lib.mdmc_render_buffers(self._ctx.handle, _dev_ptr(vertices), _dev_ptr(indices),
                                                          _stream_handle(stream)))
        return vertices, indices

    def write_obj(self, path):
        """Mesh::writeToFile, Mesh.cu:446-510"""
        self._ctx.check(self._ctx.lib.mdmc_write_obj(self._ctx.handle, str(path).encode()))

    def color_faces(self, stream=None):
        """FaceColoring::colorFaces (OriginalDMC/src/FaceColoring.cu:116-141) on
        the last run's mesh: face colors 24 -> 5, in place."""
        self._ctx.check(self._ctx.lib.mdmc_color_faces(self._ctx.handle, _stream_handle(stream)))

    def run_standard_mc(self, iso_value, grid, stream=None):
        """Standard Marching Cubes of the older CLI version (standard_mc,
        OriginalDMC/src/DualMarchingCubes.cu:201-328) on the same grid view as
        run(); leaves the DMC mesh of the last run() as it was.  Returns host
        arrays (positions [V, 3], normals [V, 3], triangles [T, 3] int32);
        the device copies stay in self.triangle_mesh until the next call."""
        g = grid.grid if isinstance(grid, UniformGrid) else grid
        self.triangle_mesh = TriangleMesh()
        self._ctx.check(self._ctx.lib.mdmc_run_standard_mc(self._ctx.handle, ctypes.byref(g), ctypes.c_float(iso_value),
                                                           ctypes.byref(self.triangle_mesh), _stream_handle(stream)))
        V, T = int(self.triangle_mesh.num_vertices), int(self.triangle_mesh.num_triangles)
        pos, nrm = np.zeros((V, 3), np.float32), np.zeros((V, 3), np.float32)
        tri = np.zeros((T, 3), np.int32)
        self._ctx.check(self._ctx.lib.mdmc_download_triangle_mesh(self._ctx.handle, _ptr(pos), _ptr(nrm), _ptr(tri),
                                                                  _stream_handle(stream)))
        return pos, nrm, tri


class BatchedDualMarchingCubes:
    """Many grids per call (mdmc_run_batch; no counterpart in the reference).
    streams = 0 lets the first run pick the number of concurrent workers."""

    def __init__(self, streams=0, **flags):
        self.lib = library()
        self.options = Options()
        self.lib.mdmc_default_options(ctypes.byref(self.options))
        for k, v in flags.items():
            setattr(self.options, k, int(v))
        self.handle = P()
        st = self.lib.mdmc_batch_create(ctypes.byref(self.handle), ctypes.byref(self.options), int(streams))
        if st != 0:
            raise MDMCError(st, "mdmc_batch_create failed")
        self.meshes = []
        self.stats = []

    def run(self, grids, iso_values, stream=None):
        n = len(grids)
        gs = (Grid * n)(*[g.grid if isinstance(g, UniformGrid) else g for g in grids])
        isos = np.ascontiguousarray(iso_values, np.float32)
        meshes = (Mesh * n)()
        stats = (Stats * n)()
        st = self.lib.mdmc_run_batch(self.handle, gs, _ptr(isos), n, meshes, stats, _stream_handle(stream))
        if st != 0:
            raise MDMCError(st, self.lib.mdmc_batch_last_error(self.handle).decode())
        self.meshes, self.stats = list(meshes), list(stats)
        return self.stats

    @property
    def streams(self):
        return int(self.lib.mdmc_batch_streams(self.handle))

    def get_halfedge_mesh(self, i):
        """Grid i's mesh of the last batch, copied to host numpy arrays."""
        ctx = self.lib.mdmc_batch_context(self.handle, int(i))
        m = self.meshes[i]
        V, F, H = int(m.num_vertices), int(m.num_faces), int(m.num_halfedges)
        out = HalfedgeMesh(np.empty((V, 3), np.float32), np.empty((V, 3), np.float32), np.empty((F, 4), np.int32),
                           np.empty((H, 4), np.int32), np.empty(F, np.int32), np.empty(F, np.uint16),
                           np.empty(V, np.int32), np.empty(V, np.uint8))
        st = self.lib.mdmc_download_mesh(ctx, _ptr(out.positions), _ptr(out.normals), _ptr(out.quads),
                                         _ptr(out.halfedges), _ptr(out.face_first_halfedge),
                                         _ptr(out.face_attributes), _ptr(out.vertex_halfedge), _ptr(out.vertex_flags),
                                         None)
        if st != 0:
            raise MDMCError(st, self.lib.mdmc_last_error(ctx).decode())
        return out

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            self.lib.mdmc_batch_destroy(h)
            self.handle = None


# SurfaceCase, UniformGrid.h:26-37
SURFACES = {"sphere": 0, "torus": 1, "two_holed_torus": 2, "four_holed_torus": 3, "genus_two": 4, "iwp": 5,
            "pw_hybrid": 6, "neovius": 7, "goursat": 8, "steiner_roman": 9}


def generate_volume(surface, dims, stream=None):
    """UniformGridHost::generateVolume (UniformGrid.inl:463-486) on the GPU:
    the implicit surface `surface` (a SURFACES name or number) sampled on
    [-1, 1]^3.  Returns (CUDA tensor [Z, Y, X] float32, origin, spacing)."""
    import torch
    lib = library()
    case = SURFACES.get(surface, surface) if isinstance(surface, str) else int(surface)
    d = np.asarray(dims, np.int32)
    out = torch.empty((int(d[2]), int(d[1]), int(d[0])), dtype=torch.float32, device="cuda")
    o, sp = np.zeros(3, np.float32), np.zeros(3, np.float32)
    st = lib.mdmc_generate_volume(int(case), _ptr(d), out.data_ptr(), _ptr(o), _ptr(sp), _stream_handle(stream))
    if st != 0:
        raise MDMCError(st, "mdmc_generate_volume failed")
    return out, o, sp


def generate_edge_case(which, stream=None):
    """UniformGridHost::generateEdgeCase (UniformGrid.inl:488-509): the 4x4x3
    NonManifoldVertex0/1 grids.  Returns (CUDA tensor, dims, origin, spacing)."""
    import torch
    lib = library()
    out = torch.empty((3, 4, 4), dtype=torch.float32, device="cuda")
    d, o, sp = np.zeros(3, np.int32), np.zeros(3, np.float32), np.zeros(3, np.float32)
    st = lib.mdmc_generate_edge_case(int(which), out.data_ptr(), _ptr(d), _ptr(o), _ptr(sp), _stream_handle(stream))
    if st != 0:
        raise MDMCError(st, "mdmc_generate_edge_case failed")
    return out, [int(x) for x in d], o, sp


def write_bin(path, samples, spacing):
    """Writes a .bin volume (int32 dims, float32 spacing, uint16 samples) that
    read_bin / UniformGridHost::readFromFile read back."""
    arr = np.ascontiguousarray(samples, np.float32)
    dims = np.asarray([arr.shape[2], arr.shape[1], arr.shape[0]], np.int32)
    st = library().mdmc_write_bin(str(path).encode(), _ptr(dims), _ptr(np.asarray(spacing, np.float32)), _ptr(arr))
    if st != 0:
        raise MDMCError(st, "cannot write %s" % path)


def case_tables():
    """(contour words [256] uint64, ambiguous [256] uint8) as built into the library."""
    lib = library()
    w = np.zeros(256, np.uint64)
    a = np.zeros(256, np.uint8)
    lib.mdmc_case_tables(_ptr(w), _ptr(a))
    return w, a


def quads_to_triangles(quads, stream=None):
    """quadrilateral_to_triangle (OriginalDMC/src/DualMarchingCubes.cu:51-60):
    CUDA int32 tensor [Q, 4] -> [2Q, 3], quad (v0, v1, v2, v3) giving
    (v0, v1, v3) and (v3, v2, v0)."""
    import torch
    q = quads.contiguous()
    out = torch.empty((2 * q.shape[0], 3), dtype=torch.int32, device=q.device)
    st = library().mdmc_quads_to_triangles(_dev_ptr(q), int(q.shape[0]), _dev_ptr(out), _stream_handle(stream))
    if st != 0:
        raise MDMCError(st, "mdmc_quads_to_triangles failed")
    return out


def mean_ratio(positions, triangles, stream=None):
    """Mean-ratio quality per triangle (QualityMeasure::mean_ratio,
    OriginalDMC/src/QualityMeasure.h:45-66) of CUDA tensors positions [V, 3]
    float32 and triangles [T, 3] int32; raises on a vertex id outside [0, V)."""
    import torch
    p, t = positions.contiguous(), triangles.contiguous()
    q = torch.empty(t.shape[0], dtype=torch.float32, device=t.device)
    bad = torch.zeros(1, dtype=torch.int32, device=t.device)
    st = library().mdmc_mean_ratio(_dev_ptr(p), int(p.shape[0]), _dev_ptr(t), int(t.shape[0]), _dev_ptr(q),
                                   _dev_ptr(bad), _stream_handle(stream))
    if st != 0:
        raise MDMCError(st, "mdmc_mean_ratio failed")
    if int(bad.item()):
        raise MDMCError(1, "triangle vertex id outside the vertex array")
    return q


class PointIndex:
    """Exact nearest-point queries against a fixed set of CUDA float32 points
    [P, 3] (mdmc_point_index_*; no counterpart in the reference): a tiled
    search on the GPU over the points in Morton order, skipping the tiles
    whose bounding box is farther than a query's best distance so far."""

    def __init__(self, points, stream=None):
        import torch
        if not points.is_cuda or points.dtype != torch.float32 or points.dim() != 2 or points.shape[1] != 3:
            raise ValueError("points must be a CUDA float32 tensor [P, 3]")
        self.lib = library()
        self.points = points.contiguous()
        self.handle = P()
        st = self.lib.mdmc_point_index_create(ctypes.byref(self.handle), self.points.data_ptr(), len(self.points),
                                              _stream_handle(stream if stream is not None
                                                             else torch.cuda.current_stream()))
        if st != 0:
            raise MDMCError(st, "mdmc_point_index_create failed")
        self._scratch = None

    def __len__(self):
        return int(self.lib.mdmc_point_index_count(self.handle))

    def nearest(self, queries, stream=None):
        """(index int64 [Q], squared distance float32 [Q]) of the nearest point to each CUDA float32 query [Q, 3]."""
        import torch
        q = queries.detach().contiguous().float()
        idx = torch.empty(len(q), dtype=torch.int32, device=q.device)
        d2 = torch.empty(len(q), dtype=torch.float32, device=q.device)
        need = 2 * len(q) + 2056  # mdmc_point_index_nearest's scratch
        if self._scratch is None or len(self._scratch) < need:
            self._scratch = torch.empty(need, dtype=torch.int64, device=q.device)
        st = self.lib.mdmc_point_index_nearest(self.handle, q.data_ptr(), len(q), idx.data_ptr(), d2.data_ptr(),
                                               self._scratch.data_ptr(),
                                               _stream_handle(stream if stream is not None
                                                              else torch.cuda.current_stream()))
        if st != 0:
            raise MDMCError(st, "mdmc_point_index_nearest failed")
        return idx.long(), d2

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            self.lib.mdmc_point_index_destroy(h)
            self.handle = None

