"""ctypes binding of libtfcuda.so and its in-tree build.

The library is built from ``transiflow_gb300/csrc/*.cu`` with nvcc for
sm_103a only and placed next to this file.  ``load()`` fails loudly when the
library is missing: there is no CPU fallback for any kernel.
"""

import ctypes
import os
import shutil
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIBNAME = 'libtfcuda.so'
LIBPATH = os.path.join(HERE, LIBNAME)
INCLUDE = os.path.join(os.path.dirname(HERE), 'include')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
# the assembly TU keeps the reference's separate multiply/add rounding
SOURCES = [('tf_assemble.cu', ['-fmad=false']), ('tf_sparse.cu', []), ('tf_nd.cu', []), ('tf_nd_panel_f32.cu', []),
           ('tf_nd_panel_f64.cu', []),
           ('tf_nd_inv.cu', []), ('tf_nd_tc.cu', []), ('tf_nd_flow.cu', []),
           ('tf_surrogate.cu', [])]

TF_MAX_BC_OPS = 24
TF_METRIC_FIELDS = 10
TF_BC_WALL = 1
TF_BC_FORCE = 2
TF_BC_FORCE_PROFILE = 3
TF_BC_PIN = 4


def _nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: set NVCC or put the CUDA toolkit on PATH')


def build(verbose=False):
    """Compile the CUDA sources (in parallel) and link libtfcuda.so in-tree."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    common = ['-std=c++17', '-O3', '-lineinfo', '-Xcompiler', '-fPIC', '-I', INCLUDE] + ARCH

    def compile_one(item):
        src, extra = item
        obj = os.path.join(BUILD, src.replace('.cu', '.o'))
        cmd = [nvcc] + common + extra + ['-c', os.path.join(CSRC, src), '-o', obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, ' '.join(cmd), res.stderr))
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIBPATH + '.tmp'
    cmd = [nvcc] + ARCH + ['-shared', '-o', tmp] + objs + ['-lcudart']
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('link failed:\n%s\n%s' % (' '.join(cmd), res.stderr))
    os.replace(tmp, LIBPATH)
    return LIBPATH


class BcOp(ctypes.Structure):
    _fields_ = [('kind', ctypes.c_int32), ('axis', ctypes.c_int32), ('high', ctypes.c_int32),
                ('var', ctypes.c_int32), ('fc', ctypes.c_double), ('ac', ctypes.c_double)]


class Problem(ctypes.Structure):
    _fields_ = [('nx', ctypes.c_int32), ('ny', ctypes.c_int32), ('nz', ctypes.c_int32),
                ('dim', ctypes.c_int32), ('dof', ctypes.c_int32), ('nonlinear', ctypes.c_int32),
                ('buoy_row', ctypes.c_int32), ('biot_row', ctypes.c_int32),
                ('visc', ctypes.c_double), ('cond', ctypes.c_double), ('biot', ctypes.c_double),
                ('d_metric', ctypes.c_void_p), ('metric_stride', ctypes.c_int32),
                ('nops', ctypes.c_int32), ('ops', BcOp * TF_MAX_BC_OPS),
                ('rossby', ctypes.c_double), ('wind', ctypes.c_double), ('asym', ctypes.c_double),
                ('d_aux', ctypes.c_void_p), ('sal', ctypes.c_double), ('d_prof', ctypes.c_void_p),
                ('prof_len', ctypes.c_int32), ('nprof', ctypes.c_int32)]


class NdPlan(ctypes.Structure):
    _fields_ = [('n', ctypes.c_int32), ('nnodes', ctypes.c_int32), ('nlevels', ctypes.c_int32),
                ('level_ptr', ctypes.c_void_p), ('max_own', ctypes.c_void_p), ('max_f', ctypes.c_void_p),
                ('d_n_own', ctypes.c_void_p), ('d_f', ctypes.c_void_p), ('d_parent', ctypes.c_void_p),
                ('d_front_off', ctypes.c_void_p), ('d_idx_off', ctypes.c_void_p), ('d_idx', ctypes.c_void_p),
                ('d_ea_off', ctypes.c_void_p), ('d_ea_map', ctypes.c_void_p),
                ('nscat', ctypes.c_int64), ('d_scat_pos', ctypes.c_void_p), ('d_scat_src', ctypes.c_void_p),
                ('scat_level_ptr', ctypes.c_void_p), ('d_piv_off', ctypes.c_void_p),
                ('d_rank', ctypes.c_void_p), ('front_elems', ctypes.c_int64), ('tc_min_front', ctypes.c_int32),
                ('tc_terms', ctypes.c_int32), ('apply_waves', ctypes.c_int32)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_SIGNATURES = {
    'tf_version': ([], _I),
    'tf_error_string': ([_I], ctypes.c_char_p),
    'tf_launch_count': ([], ctypes.c_longlong),
    'tf_launch_count_reset': ([], None),
    'tf_stream_create': ([_P], _I),
    'tf_stream_destroy': ([_P], _I),
    'tf_stencil_layout': ([_I, _I, _P, _P], _I),
    'tf_stencil_pattern': ([_P, _P, _P, _P], _I),
    'tf_assemble': ([_P, _P, _P, _P, _P], _I),
    'tf_mass_diag': ([_P, _P, _P], _I),
    'tf_csr_compact': ([_I, _P, _P, _P, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
    'tf_csr_compact_workspace_bytes': ([_I], ctypes.c_size_t),
    'tf_gauge_values': ([_I, _P, _P, _P, _I, _P, _P], _I),
    'tf_spmv_f64': ([_I, _P, _P, _P, _P, _P, _D, _D, _P], _I),
    'tf_nd_tc_update_f32': ([_P, _I, _I, _I, _P, _P, _P], _I),
    'tf_equilibrate': ([_I, _P, _P, _P, _P, _P, _P, _P], _I),
    'tf_vec_mul': ([_I, _P, _P, _P, _P], _I),
    'tf_spmv_f32': ([_I, _P, _P, _P, _P, _P, _D, _D, _P], _I),
    'tf_diag_axpy': ([_I, _D, _P, _P, _P, _P], _I),
    'tf_add_diagonal': ([_I, _P, _P, _P, _D, _P, _P], _I),
    'tf_vec_mdot': ([_I, _I, _P, ctypes.c_longlong, _P, _P, _P, ctypes.c_size_t, _P], _I),
    'tf_vec_mdot_workspace_bytes': ([_I, _I], ctypes.c_size_t),
    'tf_vec_mdot_noalloc': ([_I, _I, _P, ctypes.c_longlong, _P, _P, _P], _I),
    'tf_vec_mgs_update': ([_I, _I, _P, ctypes.c_longlong, _P, _P, _P], _I),
    'tf_vec_axpby': ([_I, _D, _P, _D, _P, _P, _P], _I),
    'tf_vec_div': ([_I, _P, _D, _P, _P], _I),
    'tf_vec_fill': ([_I, _D, _P, _P], _I),
    'tf_vec_scale_rsqrt': ([_I, _P, _P, _P], _I),
    'tf_vec_to_f32': ([_I, _P, _P, _P], _I),
    'tf_nd_factor_f64': ([_P, _P, _P, _P, _P, _P], _I),
    'tf_nd_factor_f32': ([_P, _P, _P, _P, _P, _P], _I),
    'tf_nd_solve_f64': ([_P, _P, _P, _P, _P], _I),
    'tf_nd_solve_f32': ([_P, _P, _P, _P, _P], _I),
    'tf_nd_invert_workspace_bytes': ([_P, _I], ctypes.c_size_t),
    'tf_nd_invert_f64': ([_P, _P, _P, ctypes.c_size_t, _P], _I),
    'tf_nd_invert_f32': ([_P, _P, _P, ctypes.c_size_t, _P], _I),
    'tf_nd_factor_inv_f64': ([_P, _P, _P, _P, _P, _P, ctypes.c_size_t, _P, _P], _I),
    'tf_nd_factor_inv_f32': ([_P, _P, _P, _P, _P, _P, ctypes.c_size_t, _P, _P], _I),
    'tf_nd_solve_inv_workspace_bytes': ([_P], ctypes.c_size_t),
    'tf_nd_solve_inv_f64': ([_P, _P, _P, _P, _P, _P], _I),
    'tf_nd_solve_inv_f32': ([_P, _P, _P, _P, _P, _P], _I),
    'tf_nd_factors_to_bf16': ([_P, _P, _P, _P], _I),
    'tf_nd_solve_inv_bf16': ([_P, _P, _P, _P, _P, _P], _I),
    'tf_nd_flow_workspace_bytes': ([_P, _I, _I], ctypes.c_size_t),
    'tf_nd_flow_prepare': ([_P, _P, ctypes.c_size_t, _I, _I, _I], _I),
    'tf_nd_solve_flow_f64': ([_P, _P, _P, _P, _P, _P], _I),
    'tf_nd_solve_flow_f32': ([_P, _P, _P, _P, _P, _P], _I),
    'tf_nd_flow_status': ([_P], _I),
    'tf_nd_flow_tasks_host': ([_I, _P, _P, _P, _I, _P, _I, _I, _P, _P, _I, _P], _I),
    'tf_sg_conv': ([_I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _I, _P], _I),
    'tf_sg_wgrad_workspace_bytes': ([_I, _I, _I], ctypes.c_size_t),
    'tf_sg_wgrad': ([_I, _I, _I, _I, _I, _P, _P, _P, _I, _P, ctypes.c_size_t, _P], _I),
    'tf_sg_loss_workspace_bytes': ([_I, _I], ctypes.c_size_t),
    'tf_sg_loss': ([_I, _I, _I, _P, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], _I),
    'tf_sg_act_grad': ([ctypes.c_longlong, _P, _P, _P, _P, _P], _I),
    'tf_sg_pack': ([_I, _I, _I, _P, _P, _P, _P, _P, _P, ctypes.c_float, ctypes.c_float, _P, _P], _I),
    'tf_sg_target': ([_I, _I, _P, _P, _P, _D, _P, _P, _P], _I),
    'tf_sg_unpack': ([_I, _I, _I, _P, _P, _P, _D, _P, _P, _P], _I),
    'tf_sg_adam': ([_I, _I, _P, _P, _P, _P, _P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                    _I, ctypes.c_float, _P, _P, _P], _I),
}

_lib = None


class CudaBackendError(RuntimeError):
    pass


def load():
    """Load libtfcuda.so from the package directory (raises if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise CudaBackendError('%s is missing: run `python -c "import __graft_entry__ as g; g.build()"` '
                               'to build the CUDA backend (there is no CPU fallback)' % LIBPATH)
    lib = ctypes.CDLL(LIBPATH)
    for name, (args, res) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


_streams = []
_streams_lock = threading.Lock()


def new_stream(device=None):
    """A torch stream over a CUDA stream of its own (tf_stream_create).
    Pooled torch streams repeat after a few dozen allocations, and two
    threads capturing and launching on one CUDA stream break each other's
    graph capture.  The streams live until the process exits: PyTorch's
    allocators keep stream handles with the memory used on them, so a
    destroyed (and later recycled) handle could be touched again."""
    import torch
    lib = load()
    handle = ctypes.c_void_p()
    check(lib.tf_stream_create(ctypes.byref(handle)), 'tf_stream_create')
    with _streams_lock:
        _streams.append(handle)
    return torch.cuda.ExternalStream(handle.value, device=device)


def exported_symbols():
    return list(_SIGNATURES)


def check(code, what=''):
    if code != 0:
        msg = load().tf_error_string(code).decode()
        raise CudaBackendError('%s failed: %s (code %d)' % (what or 'libtfcuda call', msg, code))
