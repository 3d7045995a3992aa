"""ctypes bindings of libfluidgrid_gb300.so (include/fluidgrid_gb300.h and
include/fluidgrid_reference.h).  The library is required: importing the
bindings raises if it has not been built -- there is no CPU fallback."""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libfluidgrid_gb300.so")

c_f = ctypes.c_float
c_u32 = ctypes.c_uint32
c_i32 = ctypes.c_int32
VP = ctypes.c_void_p


class float2(ctypes.Structure):
    _fields_ = [("x", c_f), ("y", c_f)]


class float3(ctypes.Structure):
    _fields_ = [("x", c_f), ("y", c_f), ("z", c_f)]


class float4(ctypes.Structure):
    _fields_ = [("x", c_f), ("y", c_f), ("z", c_f), ("w", c_f)]


class int3(ctypes.Structure):
    _fields_ = [("x", c_i32), ("y", c_i32), ("z", c_i32)]


class fgr_common_fluid_params(ctypes.Structure):
    """Layout of the reference's CommonFluidParams (ApplicationData.cuh:46-67)."""
    _fields_ = [("cell_size", float3), ("bucket_size", int3), ("keyBits", c_u32), ("kernel_radius", c_f),
                ("kernel_radius_squared", c_f), ("pointRadius", c_f), ("pointScale", c_f),
                ("velocity_limit", c_f), ("volume_min", float3), ("volume_max", float3),
                ("global_external_force", float3), ("simulation_scale", c_f), ("deltaTimeIntegration", c_f),
                ("fluid_to_srb_relation", int3)]


class fgr_kernels_cache(ctypes.Structure):
    _fields_ = [("kPoly6", c_f), ("kSpikyGradient", c_f), ("kViscosityLaplacian", c_f)]


class fg_body_desc(ctypes.Structure):
    _fields_ = [("n_spheres", c_u32), ("local_spheres", VP), ("mass", c_f), ("position", c_f * 3),
                ("orientation", c_f * 4), ("inv_inertia", c_f * 9)]


class fg_scene_desc(ctypes.Structure):
    _fields_ = [("n_particles", c_u32), ("positions", VP), ("velocities", VP), ("cell_size", c_f * 3),
                ("bucket_size", c_i32 * 3), ("kernel_radius", c_f), ("velocity_limit", c_f),
                ("volume_min", c_f * 3), ("volume_max", c_f * 3), ("gravity", c_f * 3),
                ("simulation_scale", c_f), ("dt", c_f), ("mass", c_f), ("rest_density", c_f),
                ("gas_constant", c_f), ("viscosity", c_f), ("wall_distance", c_f), ("wall_stiffness", c_f),
                ("wall_damping", c_f), ("noslip_min", c_f * 3), ("noslip_max", c_f * 3),
                ("friction_kinetic", c_f), ("friction_static", c_f), ("n_bodies", c_u32),
                ("bodies", ctypes.POINTER(fg_body_desc)), ("fluid_radius", c_f), ("rb_radius", c_f),
                ("rb_bucket_size", c_i32 * 3), ("fluid_to_rb_relation", c_i32 * 3),
                ("rb_to_fluid_relation", c_i32 * 3), ("contact_kspring", c_f), ("contact_kdamping", c_f),
                ("fluid_contact_eps", c_f), ("rb_contact_eps", c_f), ("rb_rb_contact", c_i32),
                ("rbrb_kspring", c_f), ("rbrb_kdamping", c_f), ("rbrb_eps", c_f), ("rb_gravity", c_f * 4),
                ("rb_velocity_limit", c_f), ("rb_dt", c_f), ("rb_volume_min", c_f * 3),
                ("rb_volume_max", c_f * 3)]


class fg_server_config(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_size_t), ("max_particles", c_u32), ("max_admit_per_step", c_u32),
                ("use_graphs", ctypes.c_int), ("grow_via_host", ctypes.c_int), ("pipeline_depth", ctypes.c_int),
                ("target_step_ms", c_f), ("head_wait_s", c_f), ("autotune_period", ctypes.c_int)]


class fg_server_step_info(ctypes.Structure):
    _fields_ = [("active_scenes", c_u32), ("admitted", c_u32), ("finished", c_u32), ("queued", c_u32),
                ("active_particles", ctypes.c_uint64), ("step_ms", c_f), ("pad_", c_f),
                ("wall_ms", ctypes.c_double), ("resident_bytes", ctypes.c_size_t)]


class fg_request_info(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int), ("steps_done", c_u32), ("steps_total", c_u32), ("n_particles", c_u32),
                ("submit_s", ctypes.c_double), ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double),
                ("resident_bytes", ctypes.c_size_t)]


class fg_server_stats_info(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_uint64), ("particle_steps", ctypes.c_uint64), ("queued", c_u32),
                ("active", c_u32), ("resident_bytes", ctypes.c_size_t), ("resident_particles", ctypes.c_uint64),
                ("device_bytes", ctypes.c_size_t)]


REQ_QUEUED, REQ_ACTIVE, REQ_DONE = 0, 1, 2

# buffer ids (fg_buffer_id)
BUFFERS = ["POS", "VEL", "KEYS_UNSORTED", "KEYS", "IDS", "START", "END", "SPOS", "SVEL", "DP",
           "RB_LOCAL", "RB_WORLD", "RB_KEYS_UNSORTED", "RB_KEYS", "RB_IDS", "RB_START", "RB_END", "RB_SPOS",
           "RB_FORCE", "RB_TORQUE", "BODY_X", "BODY_V", "BODY_Q", "BODY_L", "BODY_FSUM", "BODY_TSUM",
           "BODY_XF", "BODY_VF", "BODY_QF", "BODY_MASS", "BODY_INV_INERTIA"]
BUF = {n: i for i, n in enumerate(BUFFERS)}

STAGE_HASH, STAGE_SORT, STAGE_RANGES, STAGE_DENSITY = 1, 2, 4, 8
STAGE_RB_GRID, STAGE_RB_CONTACT, STAGE_FORCES, STAGE_BODIES = 16, 32, 64, 128
STAGE_ALL = 255

# fg_world_run_stage: one stage of a step at a time, in this order
RUN = {"neighbourhood": 1, "density": 2, "rb_grid": 3, "rb_from_fluid": 4, "rb_from_rb": 5, "forces": 6,
       "body_sums": 7, "body_integrate": 8, "integrate": 9}
RUN_WITH_CONTACT = 1

OPTIONS = {"neighbor_list": 1, "target_order": 2, "order_period": 3, "digit_bits": 4, "kernel": 5,
           "autotune_period": 6, "autotune_kernels": 7, "list_cap": 8, "ctas_per_sm": 10,
           "autotune_tiles": 11, "list_autogrow": 12, "graph_steps": 13, "one_pass_sort": 14, "block_size": 16,
           "runs_per_cta": 17}
NUM_KERNELS = 3

STATUS = {0: "FG_OK", 1: "FG_E_INVALID", 2: "FG_E_CUDA", 3: "FG_E_OOM", 4: "FG_E_BUDGET", 5: "FG_E_NONFINITE",
          6: "FG_E_TIMEOUT", 7: "FG_E_STATE", 8: "FG_E_UNSUPPORTED", 9: "FG_E_NOLIB"}

# every symbol the two public headers declare
C_ABI_SYMBOLS = [
    "fg_scene_desc_defaults", "fg_world_create", "fg_world_destroy", "fg_world_step", "fg_world_run_stage",
    "fg_world_sync",
    "fg_world_check", "fg_world_upload", "fg_world_download", "fg_world_scene_upload", "fg_world_scene_download",
    "fg_world_particles", "fg_world_scenes", "fg_world_spheres", "fg_world_bodies", "fg_world_scene_layout",
    "fg_world_buffer", "fg_world_set_stages", "fg_world_set_fused_integrate", "fg_world_set_sort_digit_bits",
    "fg_world_set_graphs", "fg_world_launches_per_step", "fg_world_kernel_launches", "fg_world_stage_profile", "fg_world_timed_steps",
    "fg_world_e2e_steps", "fg_host_alloc", "fg_host_free", "fg_set_device", "fg_probe_fp32_peak",
    "fg_sort_pairs_noalloc", "fg_selftest_bounded_wait", "fg_world_set_option", "fg_world_get_option", "fg_world_tuning_stats",
    "fg_world_counters", "fg_world_list_overflows", "fg_world_timed_blocks", "fg_world_diagnostics", "fg_server_config_defaults", "fg_server_create",
    "fg_server_destroy", "fg_server_submit", "fg_server_step", "fg_server_request", "fg_server_result",
    "fg_server_stats", "fg_server_active",
    "fg_memcpy_d2h", "fg_memcpy_h2d",
    "fg_device_synchronize", "fg_last_error", "fg_version"]
REFERENCE_SYMBOLS = [
    "gCalcHashKey", "gCalcHashKeyWithOffset", "gFindCellOffsetOrderingPosVel", "gFindCellOffsetOrderingPos",
    "gCalcMassDensity", "gInitializeKernelParams", "gSPHCalculateForces", "gSPHIntegrate",
    "gInitializeCommonFluidParams", "gSPHCalculateForcesWithSRB", "gSort", "gCalculateRigidBodyForcesFromRB",
    "gCalculateRigidBodyForcesFromFluids", "gCopyRBDataToParticle", "gReorderForceTorque", "gAddForceTorque",
    "gIntegrateRB", "fgc_sort_pairs", "fgc_segmented_scan_float4", "fgc_last_status"]

_lib = None


class FluidGridError(RuntimeError):
    pass


def lib_path():
    return LIB_PATH


def load():
    """Load the CUDA library; raises FluidGridError if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FluidGridError("libfluidgrid_gb300.so is not built (run `python -m fluidgrid_gb300.build`); "
                             "there is no CPU fallback")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    L.fg_scene_desc_defaults.argtypes = [P(fg_scene_desc)]
    L.fg_scene_desc_defaults.restype = None
    L.fg_world_create.argtypes = [P(fg_scene_desc), c_u32, VP, P(VP)]
    for n in ("fg_world_destroy", "fg_world_sync", "fg_world_check"):
        getattr(L, n).argtypes = [VP]
    L.fg_world_step.argtypes = [VP, c_u32]
    L.fg_world_run_stage.argtypes = [VP, ctypes.c_int, ctypes.c_int]
    L.fg_world_upload.argtypes = [VP, VP, VP]
    L.fg_world_download.argtypes = [VP, VP, VP]
    L.fg_world_scene_upload.argtypes = [VP, c_u32, VP, VP]
    L.fg_world_scene_download.argtypes = [VP, c_u32, VP, VP]
    for n in ("fg_world_particles", "fg_world_scenes", "fg_world_spheres", "fg_world_bodies",
              "fg_world_launches_per_step"):
        getattr(L, n).argtypes = [VP]
        getattr(L, n).restype = c_u32
    L.fg_world_kernel_launches.argtypes = [VP, P(ctypes.c_uint64)]
    L.fg_world_scene_layout.argtypes = [VP, c_u32, P(c_u32)]
    L.fg_world_buffer.argtypes = [VP, ctypes.c_int, P(VP), P(ctypes.c_size_t)]
    L.fg_world_set_stages.argtypes = [VP, c_u32]
    L.fg_world_set_fused_integrate.argtypes = [VP, ctypes.c_int]
    L.fg_world_set_sort_digit_bits.argtypes = [VP, c_u32]
    L.fg_world_set_graphs.argtypes = [VP, ctypes.c_int]
    L.fg_world_stage_profile.argtypes = [VP, ctypes.c_size_t, P(c_f)]
    L.fg_world_timed_steps.argtypes = [VP, c_u32, ctypes.c_size_t, P(c_f)]
    L.fg_world_timed_blocks.argtypes = [VP, c_u32, c_u32, ctypes.c_size_t, P(c_f)]
    L.fg_world_diagnostics.argtypes = [VP, P(ctypes.c_double)]
    L.fg_world_e2e_steps.argtypes = [VP, c_u32, VP, VP, VP, VP, P(c_f)]
    L.fg_host_alloc.argtypes = [ctypes.c_size_t]
    L.fg_host_alloc.restype = VP
    L.fg_host_free.argtypes = [VP]
    L.fg_set_device.argtypes = [ctypes.c_int]
    L.fg_probe_fp32_peak.argtypes = [P(c_f)]
    L.fg_sort_pairs_noalloc.argtypes = [VP, VP, c_u32, c_u32, VP]
    L.fg_selftest_bounded_wait.argtypes = [c_u32, P(c_u32)]
    L.fg_world_set_option.argtypes = [VP, ctypes.c_int, ctypes.c_int]
    L.fg_world_get_option.argtypes = [VP, ctypes.c_int, P(ctypes.c_int)]
    L.fg_world_tuning_stats.argtypes = [VP, P(c_u32), P(c_f)]
    L.fg_world_counters.argtypes = [VP, ctypes.c_int, P(ctypes.c_uint64), P(ctypes.c_uint64)]
    L.fg_world_list_overflows.argtypes = [VP, ctypes.c_int, P(ctypes.c_uint64)]
    L.fg_server_config_defaults.argtypes = [P(fg_server_config)]
    L.fg_server_config_defaults.restype = None
    L.fg_server_create.argtypes = [P(fg_server_config), VP, P(VP)]
    L.fg_server_destroy.argtypes = [VP]
    L.fg_server_destroy.restype = None
    L.fg_server_submit.argtypes = [VP, P(fg_scene_desc), c_u32, P(ctypes.c_uint64)]
    L.fg_server_step.argtypes = [VP, P(fg_server_step_info)]
    L.fg_server_request.argtypes = [VP, ctypes.c_uint64, P(fg_request_info)]
    L.fg_server_result.argtypes = [VP, ctypes.c_uint64, VP, VP, ctypes.c_int]
    L.fg_server_stats.argtypes = [VP, P(fg_server_stats_info)]
    L.fg_server_active.argtypes = [VP, P(ctypes.c_uint64), c_u32, P(c_u32)]
    L.fg_memcpy_d2h.argtypes = [VP, VP, ctypes.c_size_t]
    L.fg_memcpy_h2d.argtypes = [VP, VP, ctypes.c_size_t]
    L.fg_last_error.restype = ctypes.c_char_p
    L.fg_version.restype = ctypes.c_char_p
    # reference-named launchers
    L.gCalcHashKey.argtypes = [VP, VP, VP, c_u32, c_u32, float3]
    L.gCalcHashKeyWithOffset.argtypes = [VP, VP, VP, VP, VP, VP, c_u32, float3, ctypes.c_int]
    L.gFindCellOffsetOrderingPosVel.argtypes = [VP] * 8 + [c_u32, c_u32]
    L.gFindCellOffsetOrderingPos.argtypes = [VP] * 6 + [c_u32, c_u32]
    L.gCalcMassDensity.argtypes = [VP] * 5 + [ctypes.c_int, c_f, c_f, c_f]
    L.gInitializeKernelParams.argtypes = [fgr_kernels_cache]
    L.gInitializeCommonFluidParams.argtypes = [fgr_common_fluid_params]
    L.gSPHCalculateForces.argtypes = [VP] * 8 + [c_u32, c_f, c_f]
    L.gSPHIntegrate.argtypes = [VP, VP, VP, c_u32, VP, VP, VP]
    L.gSPHCalculateForcesWithSRB.argtypes = ([VP] * 8 + [c_u32, c_f, c_f, c_f, int3, c_f, float3, c_f, c_f] +
                                             [VP, VP, VP, c_u32, VP, VP, VP, VP, c_u32, ctypes.c_bool,
                                              ctypes.c_bool])
    L.gSort.argtypes = [VP, VP, ctypes.c_int]
    L.gCalculateRigidBodyForcesFromRB.argtypes = ([VP] * 7 + [c_u32, float3, c_f, ctypes.c_int, ctypes.c_int] +
                                                  [VP, VP, VP, c_f, c_f, ctypes.c_int])
    L.gCalculateRigidBodyForcesFromFluids.argtypes = ([VP] * 7 + [c_u32, float3, c_f, ctypes.c_int] +
                                                      [VP, VP, VP, VP, c_f, float3, c_u32, int3, c_f, c_f])
    L.gCopyRBDataToParticle.argtypes = [VP, VP, VP, ctypes.c_size_t]
    L.gReorderForceTorque.argtypes = [VP] * 5 + [c_u32]
    L.gAddForceTorque.argtypes = [VP] * 6 + [ctypes.c_size_t]
    L.gIntegrateRB.argtypes = [VP, VP, VP, VP, ctypes.c_size_t, c_f, float4, float3, float3, VP, VP, VP, VP, VP, c_f]
    L.fgc_sort_pairs.argtypes = [VP, VP, c_u32, c_u32]
    L.fgc_segmented_scan_float4.argtypes = [VP, VP, VP, c_u32]
    L.fgc_last_status.restype = ctypes.c_int
    _lib = L
    return L


def check(status, what=""):
    if status != 0:
        msg = load().fg_last_error().decode(errors="replace")
        raise FluidGridError("%s failed: %s (%s)" % (what, STATUS.get(status, status), msg))
