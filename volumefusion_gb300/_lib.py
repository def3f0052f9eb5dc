"""ctypes binding of libafx.so (the sm_103a CUDA library, C ABI in include/afx/afx.h).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libafx.so")

vp = C.c_void_p
i32 = C.c_int
i64 = C.c_long
f32 = C.c_float
f64 = C.c_double
sz = C.c_size_t


class PrepParams(C.Structure):
    _fields_ = [("K", f32 * 9), ("depth_threshold", f32), ("bilateral", i32), ("bilateral_r", i32), ("sigma_i", f32),
                ("sigma_s", f32), ("bilateral_thr", f32), ("excl_angle_lo", f32), ("excl_angle_hi", f32)]


class CameraDistortion(C.Structure):
    """af::CameraDistortion (include/af/CameraModel.h:21-33)."""
    _fields_ = [("k1", f32), ("k2", f32), ("k3", f32), ("k4", f32), ("k5", f32), ("k6", f32), ("codx", f32),
                ("cody", f32), ("p1", f32), ("p2", f32), ("is_distorted", i32)]


class FusionParams(C.Structure):
    _fields_ = [("width", i32), ("height", i32), ("K", f32 * 9), ("dims", i32 * 3), ("volume_size", f32 * 3),
                ("delta", f32), ("depth_threshold", f32), ("bilateral", i32), ("bilateral_r", i32), ("sigma_i", f32),
                ("sigma_s", f32), ("bilateral_thr", f32), ("excl_angle_lo", f32), ("excl_angle_hi", f32),
                ("graph_radius", f32), ("knn", i32), ("kreg", i32), ("update_graph", i32), ("icp_iterations", i32),
                ("gn_iterations", i32), ("lambda_depth", f32), ("lambda_reg", f32), ("energy_min_step", f32),
                ("corr_thresh", f32), ("solver", i32), ("pcg_iterations", i32), ("pcg_tol", f64), ("integrate", i32),
                ("extract_mesh", i32), ("node_capacity", i32), ("mesh_capacity", i64), ("triangle_capacity", i64),
                ("precision", i32), ("warp_mesh", i32), ("blend", i32), ("distortion", CameraDistortion)]


class FrameStats(C.Structure):
    _fields_ = [("frame", i32), ("n_nodes", i32), ("new_nodes", i32), ("mesh_points", C.c_uint),
                ("correspondences", C.c_uint), ("gn_iterations_done", i32), ("energy", f64),
                ("mesh_vertices", C.c_uint), ("mesh_faces", C.c_uint), ("error", i32)]


class ServerResult(C.Structure):
    _fields_ = [("session_id", i32), ("tag", C.c_uint64), ("latency_ms", f64), ("stats", FrameStats)]


class ServerCounters(C.Structure):
    _fields_ = [("opens_fresh", C.c_long), ("opens_reused", C.c_long), ("evictions", C.c_long),
                ("idle_sessions", i32), ("idle_bytes", C.c_size_t), ("submits", C.c_long), ("polls", C.c_long),
                ("results", C.c_long), ("open_ms", f64), ("staging_ms", f64), ("enqueue_ms", f64), ("poll_ms", f64)]


SIGNATURES = {
    "afx_status_string": (C.c_char_p, [i32]),
    "afx_version": (i32, []),
    "afx_last_cuda_error": (i32, []),
    "afx_depth_from_mm": (i32, [vp, vp, i64, vp]),
    "afx_filter_depth": (i32, [vp, i64, f32, vp]),
    "afx_filter_depth_fill": (i32, [vp, i64, f32, f32, vp]),
    "afx_fill_f32": (i32, [vp, i64, f32, vp]),
    "afx_bilateral_filter": (i32, [vp, vp, i32, i32, i32, f64, f64, f32, vp]),
    "afx_depth_to_mesh": (i32, [vp, vp, i32, i32, vp, vp]),
    "afx_depth_vertices_normals": (i32, [vp, vp, i32, i32, f32, f32, vp]),
    "afx_remove_depth_without_normals": (i32, [vp, vp, vp, i32, i32, vp]),
    "afx_frame_prep": (i32, [vp, i32, i32, C.POINTER(PrepParams), vp, vp, vp, vp, vp]),
    "afx_integrate_tsdf": (i32, [vp, vp, vp, i32, i32, f32, vp, vp, vp, vp, vp, vp, vp]),
    "afx_tsdf_knn": (i32, [vp, vp, vp, vp, vp, i32, vp, vp, vp, vp, i32, vp, sz, vp]),
    "afx_tsdf_knn_workspace_size": (sz, [vp, i32, vp]),
    "afx_tsdf_warp_weights": (i32, [vp, vp, vp, vp, vp, i64, i32, vp]),
    "afx_tsdf_vertices": (i32, [vp, vp, vp, vp, vp]),
    "afx_warp_tsdf": (i32, [vp, vp, vp, vp, vp, i64, i32, vp]),
    "afx_count_collisions": (i32, [vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "afx_integrate_warped_tsdf": (i32, [vp, vp, vp, vp, vp, vp, i32, i32, f32, vp, vp, vp, vp, vp, vp, vp]),
    "afx_marching_cubes_points": (i32, [vp, vp, i64, vp, vp, vp, vp, vp, f32, vp]),
    "afx_marching_cubes_mesh": (i32, [vp, vp, i64, vp, vp, i64, vp, vp, vp, vp, vp, f32, vp]),
    "afx_sort_unique_points": (i32, [vp, vp, i64, vp, sz, vp]),
    "afx_sort_unique_points_workspace_size": (sz, [i64]),
    "afx_sort_unique_volume_points_workspace_size": (sz, [i64, vp]),
    "afx_sort_unique_volume_points": (i32, [vp, vp, i64, vp, vp, vp, vp, sz, vp]),
    "afx_extract_point_cloud": (i32, [vp, vp, i64, vp, vp, vp, vp, vp, f32, vp, sz, vp]),
    "afx_translate": (i32, [vp, vp, i64, vp, vp]),
    "afx_build_graph": (i32, [vp, vp, vp, vp, i32, vp, vp, i64, i32, f32, vp, sz, vp]),
    "afx_build_graph_workspace_size": (sz, [i64, i32]),
    "afx_knn": (i32, [vp, vp, vp, vp, i32, vp, vp, i64, i32, i32, vp]),
    "afx_filter_disconnected": (i32, [vp, vp, vp, i32, i32, vp, vp]),
    "afx_warp_weights": (i32, [vp, vp, vp, vp, vp, i64, i32, vp, vp]),
    "afx_warp": (i32, [vp, vp, vp, vp, vp, vp, i64, i32, vp]),
    "afx_warp_dqb": (i32, [vp, vp, vp, vp, vp, vp, i64, i32, vp]),
    "afx_correspondences": (i32, [vp, vp, i64, vp, vp, i64, vp, vp, i32, i32, vp, f32, vp, sz, vp]),
    "afx_correspondences_workspace_size": (sz, [i64]),
    "afx_correspondences_static": (i32, [vp, vp, i64, vp, vp, i64, vp, vp, i32, i32, vp, f32, vp]),
    "afx_gn_create": (i32, [i64, i32, i32, i32, C.POINTER(vp)]),
    "afx_gn_destroy": (i32, [vp]),
    "afx_gn_build": (i32, [vp] + [vp] * 13 + [f32, f32, vp]),
    "afx_gn_export": (i32, [vp, i32, vp, vp, vp, vp, vp]),
    "afx_gn_solve": (i32, [vp, vp, i32, C.c_double, vp]),
    "afx_update_transforms": (i32, [vp, vp, vp, i32, vp]),
    "afx_fusion_set_graphs": (i32, [vp, i32]),
    "afx_fusion_graph_count": (i32, [vp]),
    "afx_fusion_set_tile": (i32, [vp, i32]),
    "afx_fusion_get_tile": (i32, [vp]),
    "afx_fusion_autotune": (i32, [vp, C.POINTER(i32), C.POINTER(C.c_float), vp]),
    "afx_batch_create": (i32, [C.POINTER(vp), i32, C.POINTER(vp)]),
    "afx_batch_destroy": (i32, [vp]),
    "afx_batch_process": (i32, [vp, C.POINTER(vp), vp]),
    "afx_batch_stats": (i32, [vp, vp, i32]),
    "afx_batch_graph_launches": (C.c_long, [vp]),
    "afx_fusion_default_params": (None, [C.POINTER(FusionParams)]),
    "afx_fusion_memory_bytes": (sz, [C.POINTER(FusionParams)]),
    "afx_fusion_stats_async": (i32, [vp, vp, vp]),
    "afx_server_create": (i32, [sz, i32, C.POINTER(vp)]),
    "afx_server_destroy": (i32, [vp]),
    "afx_server_open": (i32, [vp, C.POINTER(FusionParams), C.POINTER(i32)]),
    "afx_server_close": (i32, [vp, i32]),
    "afx_server_submit": (i32, [vp, i32, vp, C.c_uint64]),
    "afx_server_poll": (i32, [vp, vp, i32, C.POINTER(i32)]),
    "afx_server_session": (vp, [vp, i32]),
    "afx_server_usage": (i32, [vp, C.POINTER(sz), C.POINTER(i32), C.POINTER(C.c_long)]),
    "afx_server_get_counters": (i32, [vp, C.POINTER(ServerCounters)]),
    "afx_fusion_create": (i32, [C.POINTER(FusionParams), C.POINTER(vp)]),
    "afx_fusion_destroy": (i32, [vp]),
    "afx_fusion_reset": (i32, [vp, vp]),
    "afx_fusion_process": (i32, [vp, vp, vp]),
    "afx_fusion_process_host": (i32, [vp, vp, vp]),
    "afx_fusion_stats": (i32, [vp, C.POINTER(FrameStats), vp]),
    "afx_fusion_tsdf": (i32, [vp, C.POINTER(vp), C.POINTER(vp)]),
    "afx_fusion_volume": (i32, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(i32)]),
    "afx_fusion_graph": (i32, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]),
    "afx_fusion_centroid": (i32, [vp, C.POINTER(vp)]),
    "afx_fusion_point_cloud": (i32, [vp, C.POINTER(vp), C.POINTER(vp)]),
    "afx_fusion_mesh": (i32, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]),
    "afx_fusion_frame_views": (i32, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]),
    "afx_fusion_volume_changed": (i32, [vp, vp]),
    "afx_fusion_support_size": (i32, [vp, C.POINTER(C.c_uint), C.POINTER(C.c_ulonglong), vp]),
    "afx_fusion_occupied_bricks": (i32, [vp, C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong), vp]),
    "afx_fusion_set_transforms": (i32, [vp, vp, i32, vp]),
    "afx_fusion_kernel_launches": (i64, [vp]),
    "afx_copy_device": (i32, [vp, vp, sz, vp]),
    "afx_integrate_tsdf_fresh": (i32, [vp, vp, vp, i32, i32, f32, vp, vp, vp, vp, vp, vp, vp]),
    "afx_rigid_stream_default_params": (None, [vp]),
    "afx_rigid_stream_create": (i32, [vp, C.POINTER(vp)]),
    "afx_rigid_stream_destroy": (i32, [vp]),
    "afx_rigid_stream_process": (i32, [vp, C.POINTER(vp), vp]),
    "afx_rigid_stream_outputs": (i32, [vp, C.POINTER(vp), C.POINTER(C.c_long), C.POINTER(vp), C.POINTER(vp),
                                       C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]),
    "afx_save_ply": (i32, [C.c_char_p, vp, C.c_long, vp, vp, C.c_long]),
    "afx_tsdf_save": (i32, [C.c_char_p, vp, vp, vp, f32, vp, vp]),
    "afx_tsdf_load_header": (i32, [C.c_char_p, vp, vp, vp, vp]),
    "afx_tsdf_load": (i32, [C.c_char_p, vp, vp, C.c_long]),
    "afx_fusion_save_volume": (i32, [vp, C.c_char_p, vp]),
    "afx_fusion_load_volume": (i32, [vp, C.c_char_p, vp]),
    "afx_fusion_save_mesh_ply": (i32, [vp, C.c_char_p, vp]),
    "afx_decode_depth_image": (i32, [vp, sz, vp, i64, C.POINTER(i32), C.POINTER(i32)]),
    "afx_decode_depth_images": (i32, [i32, vp, vp, vp, vp, vp, vp, vp, i32]),
    "afx_depth_file_name": (i32, [C.c_char_p, i64, C.c_char_p, sz]),
    "afx_read_depth_frame": (i32, [C.c_char_p, i64, vp, i64, C.POINTER(i32), C.POINTER(i32)]),
    "afx_undistort_map": (i32, [vp, i32, i32, vp, vp, i32, vp]),
    "afx_undistort_depth": (i32, [vp, vp, i32, i32, vp, i32, vp]),
    "afx_xy_lookup_table": (i32, [vp, i32, i32, vp, vp, vp]),
    "afx_unproject_points": (i32, [vp, vp, vp, vp, i64, vp, vp, vp]),
    "afx_project_points": (i32, [vp, vp, vp, i64, vp, vp, vp]),
    "afx_fill_j_depth": (i32, [vp, f32, C.c_uint, C.c_uint, vp, C.c_uint, vp, vp, vp, i32, vp, vp]),
    "afx_fill_j_mreg": (i32, [vp, f32, C.c_uint, C.c_uint, vp, C.c_uint, vp, i32, vp]),
    "afx_fill_r_depth": (i32, [vp, f32, vp, C.c_uint, vp, vp, vp, vp]),
    "afx_fill_r_mreg": (i32, [vp, f32, vp, vp, C.c_uint, vp, i32, vp]),
    "afx_jtj_contrib_workspace_size": (sz, [i64]),
    "afx_jtj_contrib_depth": (i32, [vp, vp, vp, vp, vp, vp, C.c_uint, vp, vp, i32, vp, sz, vp]),
    "afx_jtj_contrib_mreg": (i32, [vp, vp, C.c_uint, vp, vp, vp, C.c_uint, vp, i32, vp, sz, vp]),
    "afx_multiply_jtj_pairs": (i32, [vp, vp, vp, C.c_uint, vp, C.c_uint, vp]),
    "afx_multiply_jtr_elems": (i32, [vp, vp, C.c_uint, vp, vp, C.c_uint, vp]),
    "afx_fill_jtj": (i32, [vp, vp, vp, C.c_uint, C.c_uint, vp]),
    "afx_fill_jtr": (i32, [vp, vp, vp, C.c_uint, vp]),
    "afx_lu_solve_workspace_size": (sz, [i32, i32]),
    "afx_lu_solve": (i32, [vp, vp, i32, i32, vp, vp, vp, sz, vp]),
    "afx_fusion_set_timing": (i32, [vp, i32]),
    "afx_fusion_stage_times": (i32, [vp, C.POINTER(f64), i32, i32]),
}

_lib = None


MAX_CAMERAS = 8


class RigidStreamParams(C.Structure):
    _fields_ = [("n_cameras", i32), ("width", i32), ("height", i32), ("K", (f32 * 9) * MAX_CAMERAS),
                ("camera_to_world", (f32 * 16) * MAX_CAMERAS), ("dims", i32 * 3), ("volume_size", f32 * 3),
                ("delta", f32), ("center", f32 * 3), ("rotation", f32 * 9), ("depth_threshold", f32),
                ("bilateral", i32), ("bilateral_r", i32), ("sigma_i", f32), ("sigma_s", f32), ("bilateral_thr", f32),
                ("triangle_capacity", i64), ("distortion", CameraDistortion * MAX_CAMERAS)]


class AfxError(RuntimeError):
    def __init__(self, status, what):
        self.status = status
        msg = lib().afx_status_string(status).decode()
        super().__init__("%s failed: %s (status %d, last CUDA error %d)" % (what, msg, status,
                                                                            lib().afx_last_cuda_error()))


def lib():
    """The loaded libafx.so.  Raises if it has not been built (python -m volumefusion_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libafx.so is missing (%s); build it with `python -m volumefusion_gb300.build`"
                               % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status, what):
    if status != 0:
        raise AfxError(status, what)
