"""ctypes binding of libcmag_sph.so (the C ABI of include/cmag_sph.h).

The library is the only compute path: if it is missing this module raises on
first use instead of falling back to anything else."""
import ctypes
import os

from ._abi import BatchGroup, SphParams

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libcmag_sph.so")

_lib = None

P = ctypes.POINTER
c_u32p = P(ctypes.c_uint32)
c_f32p = P(ctypes.c_float)
c_sys = ctypes.c_void_p
c_bat = ctypes.c_void_p
c_u32 = ctypes.c_uint32
c_i32 = ctypes.c_int32

# every symbol the header declares, with its ctypes signature
SIGNATURES = {
    "cmag_version": ([], ctypes.c_char_p),
    "cmag_sph_params_size": ([], ctypes.c_size_t),
    "cmag_last_error": ([], ctypes.c_char_p),
    "cmag_system_last_error": ([c_sys], ctypes.c_char_p),
    "cmag_dambreak_default_params": ([c_u32p, ctypes.c_int32, c_u32p, ctypes.c_float, P(SphParams)], ctypes.c_int),
    "cmag_poiseuille_default_params": ([c_u32p, ctypes.c_int32, c_u32p, ctypes.c_float, P(SphParams)], ctypes.c_int),
    "cmag_peristalsis_default_params": ([ctypes.c_float, c_u32p, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                         c_f32p, ctypes.c_int32, c_u32p, ctypes.c_float, P(SphParams)], ctypes.c_int),
    "cmag_reference_particle_count": ([P(SphParams), c_u32p], ctypes.c_int),
    "cmag_dambreak3d_particle_count": ([c_u32p, c_u32p, ctypes.c_uint32, c_u32p], ctypes.c_int),
    "cmag_reference_scene": ([P(SphParams), c_f32p, ctypes.c_uint32], ctypes.c_int),
    "cmag_peristalsis_mass_sum": ([P(SphParams), c_f32p, ctypes.c_uint32, c_f32p], ctypes.c_int),
    "cmag_dambreak3d_scene_host": ([P(SphParams), c_u32p, ctypes.c_uint32, ctypes.c_float,
                                    ctypes.c_uint64, c_f32p, ctypes.c_uint32], ctypes.c_int),
    "cmag_system_create": ([P(SphParams), ctypes.c_uint32, P(c_sys)], ctypes.c_int),
    "cmag_system_destroy": ([c_sys], ctypes.c_int),
    "cmag_system_reset": ([c_sys], ctypes.c_int),
    "cmag_dambreak3d_scene": ([c_sys, c_u32p, ctypes.c_uint32, ctypes.c_float, ctypes.c_uint64], ctypes.c_int),
    "cmag_system_update": ([c_sys], ctypes.c_int),
    "cmag_system_update_dt": ([c_sys, ctypes.c_float], ctypes.c_int),
    "cmag_system_update_n": ([c_sys, ctypes.c_uint32], ctypes.c_int),
    "cmag_system_timed_update": ([c_sys, ctypes.c_uint32, c_f32p], ctypes.c_int),
    "cmag_system_run_stages": ([c_sys, ctypes.c_int32], ctypes.c_int),
    "cmag_system_set_array": ([c_sys, ctypes.c_int32, c_f32p, ctypes.c_uint32, ctypes.c_uint32], ctypes.c_int),
    "cmag_system_get_array": ([c_sys, ctypes.c_int32, c_f32p, ctypes.c_uint32, ctypes.c_uint32], ctypes.c_int),
    "cmag_batch_set_wall_cache": ([c_bat, ctypes.c_int32], ctypes.c_int),
    "cmag_batch_get_wall_cache": ([c_bat, P(ctypes.c_int32)], ctypes.c_int),
    "cmag_system_set_wall_cache": ([c_sys, ctypes.c_int32], ctypes.c_int),
    "cmag_system_get_wall_cache": ([c_sys, P(ctypes.c_int32)], ctypes.c_int),
    "cmag_system_set_arrays": ([c_sys, ctypes.c_uint32, P(ctypes.c_int32), P(c_f32p)], ctypes.c_int),
    "cmag_system_get_arrays": ([c_sys, ctypes.c_uint32, P(ctypes.c_int32), P(c_f32p)], ctypes.c_int),
    "cmag_system_get_uint_array": ([c_sys, ctypes.c_int32, c_u32p, ctypes.c_uint32, ctypes.c_uint32], ctypes.c_int),
    "cmag_system_device_array": ([c_sys, ctypes.c_int32], ctypes.c_void_p),
    "cmag_system_num_particles": ([c_sys, c_u32p], ctypes.c_int),
    "cmag_system_num_grid_cells": ([c_sys, P(ctypes.c_uint64)], ctypes.c_int),
    "cmag_system_elapsed_time": ([c_sys, c_f32p], ctypes.c_int),
    "cmag_system_get_params": ([c_sys, P(SphParams)], ctypes.c_int),
    "cmag_system_set_params": ([c_sys, P(SphParams)], ctypes.c_int),
    "cmag_dambreak_change_right_boundary": ([c_sys], ctypes.c_int),
    "cmag_dambreak_remove_right_boundary": ([c_sys], ctypes.c_int),
    "cmag_poiseuille_change_gravity": ([c_sys], ctypes.c_int),
    "cmag_peristalsis_phase": ([c_sys, c_f32p, c_f32p, c_f32p, P(ctypes.c_int32)], ctypes.c_int),
    "cmag_system_set_elapsed_time": ([c_sys, ctypes.c_float], ctypes.c_int),
    "cmag_peristalsis_set_phase": ([c_sys, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_int32], ctypes.c_int),
    "cmag_system_fluid_extent": ([c_sys, c_f32p, c_f32p], ctypes.c_int),
    "cmag_system_fluid_sum": ([c_sys, ctypes.c_int32, P(ctypes.c_double), c_u32p], ctypes.c_int),
    "cmag_system_set_stream": ([c_sys, ctypes.c_void_p], ctypes.c_int),
    "cmag_system_stream": ([c_sys], ctypes.c_void_p),
    "cmag_system_set_graphs": ([c_sys, ctypes.c_int32], ctypes.c_int),
    "cmag_system_synchronize": ([c_sys], ctypes.c_int),
    "cmag_system_device_error_bits": ([c_sys, c_u32p], ctypes.c_int),
    "cmag_system_set_groups": ([c_sys, ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
    "cmag_system_get_groups": ([c_sys, P(ctypes.c_int32), P(ctypes.c_int32)], ctypes.c_int),
    "cmag_system_autotune": ([c_sys, ctypes.c_int32], ctypes.c_int),
    "cmag_system_set_neighbor_lists": ([c_sys, ctypes.c_int32], ctypes.c_int),
    "cmag_system_get_neighbor_lists": ([c_sys, P(ctypes.c_int32), c_u32p], ctypes.c_int),
    "cmag_system_set_verlet": ([c_sys, ctypes.c_float], ctypes.c_int),
    "cmag_system_get_verlet": ([c_sys, c_f32p, c_u32p], ctypes.c_int),
    "cmag_system_set_stage_timing": ([c_sys, ctypes.c_int32], ctypes.c_int),
    "cmag_system_stage_times": ([c_sys, c_f32p, c_u32p], ctypes.c_int),
    "cmag_sort_particles": ([c_u32p, c_u32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p], ctypes.c_int),
    "cmag_sort_particles_noalloc": ([c_u32p, c_u32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p],
                                    ctypes.c_int),
    "cmag_sort_particles_noalloc_error": ([], ctypes.c_char_p),
    "cmag_testing_set_sort_spin_limit": ([ctypes.c_int32], ctypes.c_int),
    "cmag_system_colors": ([c_sys, c_f32p], ctypes.c_int),
    "cmag_system_render_ppm": ([c_sys, ctypes.c_char_p, c_u32, c_u32], ctypes.c_int),
    # batches
    "cmag_batch_create": ([P(SphParams), c_u32p, c_u32, P(c_bat)], ctypes.c_int),
    "cmag_batch_destroy": ([c_bat], ctypes.c_int),
    "cmag_batch_num_scenes": ([c_bat, c_u32p], ctypes.c_int),
    "cmag_batch_num_particles": ([c_bat, c_u32p], ctypes.c_int),
    "cmag_batch_scene_range": ([c_bat, c_u32, c_u32p, c_u32p], ctypes.c_int),
    "cmag_batch_reset": ([c_bat], ctypes.c_int),
    "cmag_batch_reset_scene": ([c_bat, c_u32], ctypes.c_int),
    "cmag_batch_set_array": ([c_bat, c_u32, c_i32, c_f32p, c_u32, c_u32], ctypes.c_int),
    "cmag_batch_get_array": ([c_bat, c_u32, c_i32, c_f32p, c_u32, c_u32], ctypes.c_int),
    "cmag_batch_set_array_all": ([c_bat, c_i32, c_f32p], ctypes.c_int),
    "cmag_batch_get_array_all": ([c_bat, c_i32, c_f32p], ctypes.c_int),
    "cmag_batch_get_uint_array": ([c_bat, c_u32, c_i32, c_u32p, c_u32, c_u32], ctypes.c_int),
    "cmag_batch_device_array": ([c_bat, c_i32], ctypes.c_void_p),
    "cmag_batch_get_params": ([c_bat, c_u32, P(SphParams)], ctypes.c_int),
    "cmag_batch_set_params": ([c_bat, c_u32, P(SphParams)], ctypes.c_int),
    "cmag_batch_update": ([c_bat], ctypes.c_int),
    "cmag_batch_update_n": ([c_bat, c_u32], ctypes.c_int),
    "cmag_batch_timed_update": ([c_bat, c_u32, c_f32p], ctypes.c_int),
    "cmag_batch_run_stages": ([c_bat, c_i32], ctypes.c_int),
    "cmag_batch_elapsed_time": ([c_bat, c_u32, c_f32p], ctypes.c_int),
    "cmag_batch_dambreak_change_right_boundary": ([c_bat, c_u32], ctypes.c_int),
    "cmag_batch_dambreak_remove_right_boundary": ([c_bat, c_u32], ctypes.c_int),
    "cmag_batch_poiseuille_change_gravity": ([c_bat, c_u32], ctypes.c_int),
    "cmag_batch_fluid_extents": ([c_bat, c_f32p, c_f32p], ctypes.c_int),
    "cmag_batch_set_stream": ([c_bat, ctypes.c_void_p], ctypes.c_int),
    "cmag_batch_stream": ([c_bat], ctypes.c_void_p),
    "cmag_batch_set_graphs": ([c_bat, c_i32, c_u32], ctypes.c_int),
    "cmag_batch_synchronize": ([c_bat], ctypes.c_int),
    "cmag_batch_device_error_bits": ([c_bat, c_u32p], ctypes.c_int),
    "cmag_batch_num_groups": ([c_bat, c_u32p], ctypes.c_int),
    "cmag_batch_group_info": ([c_bat, c_u32, P(BatchGroup)], ctypes.c_int),
    "cmag_batch_scene_group": ([c_bat, c_u32, c_u32p], ctypes.c_int),
    "cmag_batch_set_group_lanes": ([c_bat, c_u32, c_i32, c_i32], ctypes.c_int),
    "cmag_batch_set_group_lists": ([c_bat, c_u32, c_i32], ctypes.c_int),
    "cmag_batch_autotune": ([c_bat, c_i32], ctypes.c_int),
    "cmag_batch_set_stage_timing": ([c_bat, c_i32], ctypes.c_int),
    "cmag_batch_stage_times": ([c_bat, c_f32p, c_u32p], ctypes.c_int),
    "cmag_batch_last_error": ([c_bat], ctypes.c_char_p),
    # learned closure
    "cmag_closure_param_count": ([], ctypes.c_size_t),
    "cmag_closure_create": ([c_f32p, P(ctypes.c_void_p)], ctypes.c_int),
    "cmag_closure_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "cmag_closure_set_params": ([ctypes.c_void_p, c_f32p], ctypes.c_int),
    "cmag_closure_get_params": ([ctypes.c_void_p, c_f32p], ctypes.c_int),
    "cmag_closure_get_bf16_params": ([ctypes.c_void_p, c_f32p], ctypes.c_int),
    "cmag_closure_set_normalization": ([ctypes.c_void_p, c_f32p, c_f32p, ctypes.c_float], ctypes.c_int),
    "cmag_closure_get_normalization": ([ctypes.c_void_p, c_f32p, c_f32p, c_f32p], ctypes.c_int),
    "cmag_closure_set_output_limit": ([ctypes.c_void_p, ctypes.c_float], ctypes.c_int),
    "cmag_closure_forward": ([ctypes.c_void_p, ctypes.c_void_p, c_u32, ctypes.c_void_p, ctypes.c_void_p],
                             ctypes.c_int),
    "cmag_closure_gradient": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_u32, c_f32p, c_f32p,
                               ctypes.c_void_p], ctypes.c_int),
    "cmag_closure_train_step": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_u32, ctypes.c_float,
                                 c_f32p, ctypes.c_void_p], ctypes.c_int),
    "cmag_closure_reset_optimizer": ([ctypes.c_void_p], ctypes.c_int),
    "cmag_closure_synchronize": ([ctypes.c_void_p], ctypes.c_int),
    "cmag_closure_last_error": ([ctypes.c_void_p], ctypes.c_char_p),
    "cmag_system_set_closure": ([c_sys, ctypes.c_void_p], ctypes.c_int),
    "cmag_system_closure_features": ([c_sys, ctypes.c_void_p], ctypes.c_int),
    "cmag_system_interpolate": ([c_sys, c_i32, ctypes.c_void_p, c_u32, ctypes.c_void_p], ctypes.c_int),
}


class CmagError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("cmag status %d: %s" % (code, msg))
        self.code = code


def lib():
    """Load the in-tree library (built by cmag_gb300.build / __graft_entry__.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libcmag_sph.so is not built (%s); run "
                              "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(rc, handle=None, batch=None, closure=None):
    if rc != 0:
        L = lib()
        if closure:
            msg = L.cmag_closure_last_error(closure)
        elif batch:
            msg = L.cmag_batch_last_error(batch)
        elif handle:
            msg = L.cmag_system_last_error(handle)
        else:
            msg = L.cmag_last_error()
        raise CmagError(rc, (msg or b"").decode(errors="replace"))
    return rc
