"""ctypes declarations of the C ABI in include/azu_gpu.h (libazu_gb300.so)."""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libazu_gb300.so")
SYNTH_PATH = os.path.join(HERE, "_build", "libazu_synth.so")

AZU_OK = 0
AZU_E_INVALID = -1
AZU_E_CUDA = -2
AZU_E_NOMEM = -3
AZU_E_TIMEOUT = -4
AZU_E_UNSUPPORTED = -5
AZU_E_STATE = -6

AZU_TSDF_FP32 = 0
AZU_TSDF_FP16 = 1
AZU_TSDF_FP16R = 2
AZU_PRE_FULL = 0
AZU_PRE_MINIMAL = 1

fp = C.POINTER(C.c_float)
vp = C.c_void_p


class VolumeParams(C.Structure):
    _fields_ = [("resolution", C.c_int), ("voxel_size", C.c_float), ("truncation", C.c_float),
                ("max_weight", C.c_float), ("origin", C.c_float * 3), ("min_depth", C.c_float),
                ("max_depth", C.c_float), ("format", C.c_int), ("color", C.c_int)]


class VolumeStats(C.Structure):
    _fields_ = [("integrated_frames", C.c_int), ("observed_voxels", C.c_int64),
                ("last_voxels_updated", C.c_int64), ("last_color_updates", C.c_int64),
                ("voxels", C.c_int64), ("total_voxels_updated", C.c_int64)]


class TrackerParams(C.Structure):
    _fields_ = [("max_iterations", C.c_int * 3), ("dist_threshold", C.c_float),
                ("angle_threshold", C.c_float), ("min_depth", C.c_float), ("max_depth", C.c_float),
                ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("precision", C.c_int)]


class IcpResult(C.Structure):
    _fields_ = [("pose", C.c_float * 16), ("error", C.c_float), ("inliers", C.c_int),
                ("converged", C.c_int), ("tracking_ok", C.c_int), ("final_step", C.c_float),
                ("information", C.c_float * 36), ("valid_live_points", C.c_int),
                ("valid_model_points", C.c_int), ("projected_points", C.c_int),
                ("dist_filtered", C.c_int), ("angle_filtered", C.c_int), ("iterations", C.c_int * 3),
                ("status", C.c_int)]


class MeshInfo(C.Structure):
    _fields_ = [("n_vertices", C.c_int64), ("n_indices", C.c_int64), ("truncated", C.c_int), ("launches", C.c_int)]


class PipelineParams(C.Structure):
    _fields_ = [("volume", VolumeParams), ("tracker", TrackerParams), ("preprocess_mode", C.c_int),
                ("min_depth", C.c_float), ("max_depth", C.c_float), ("input_is_mm", C.c_int),
                ("use_graph", C.c_int), ("width", C.c_int), ("height", C.c_int)]


class FrameResult(C.Structure):
    _fields_ = [("pose", C.c_float * 16), ("icp", IcpResult), ("quality", C.c_int),
                ("integrated", C.c_int), ("frame_index", C.c_int)]


class BatchScene(C.Structure):
    _fields_ = [("volume", VolumeParams), ("tracker", TrackerParams), ("width", C.c_int), ("height", C.c_int),
                ("min_depth", C.c_float), ("max_depth", C.c_float)]


# name -> (restype, argtypes)
SIGNATURES = {
    "azu_last_error": (C.c_char_p, []),
    "azu_version": (C.c_char_p, []),
    "azu_select_device": (C.c_int, [C.c_size_t, C.POINTER(C.c_int)]),
    # volume
    "azu_volume_create": (C.c_int, [C.c_int, C.POINTER(VolumeParams), vp, C.POINTER(vp)]),
    "azu_volume_destroy": (C.c_int, [vp]),
    "azu_volume_reset": (C.c_int, [vp]),
    "azu_volume_set_params": (C.c_int, [vp, C.POINTER(VolumeParams)]),
    "azu_volume_get_params": (C.c_int, [vp, C.POINTER(VolumeParams)]),
    "azu_volume_integrate": (C.c_int, [vp, vp, vp, fp, C.c_float, C.c_float, C.c_float, C.c_float,
                                       C.c_int, C.c_int, C.c_float, C.c_float]),
    "azu_volume_integrate_host": (C.c_int, [vp, vp, vp, fp, C.c_float, C.c_float, C.c_float, C.c_float,
                                            C.c_int, C.c_int, C.c_float, C.c_float]),
    "azu_volume_raycast": (C.c_int, [vp, fp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                                     vp, vp, vp]),
    "azu_volume_get_stats": (C.c_int, [vp, C.POINTER(VolumeStats)]),
    "azu_volume_download": (C.c_int, [vp, vp, vp, vp]),
    "azu_volume_upload": (C.c_int, [vp, vp, vp, vp]),
    "azu_volume_device_voxels": (vp, [vp]),
    "azu_volume_set_free_space_skipping": (C.c_int, [vp, C.c_int]),
    "azu_volume_voxels_changed": (C.c_int, [vp]),
    "azu_volume_raycast_many": (C.c_int, [vp, fp, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                                          C.c_int, vp, vp]),
    "azu_volume_point_cloud": (C.c_int, [vp, vp, vp, C.c_int64, C.POINTER(C.c_int64)]),
    "azu_volume_render_depth": (C.c_int, [vp, fp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, vp]),
    "azu_volume_depth_backward": (C.c_int, [vp, fp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                                            vp, C.c_float, vp, vp, vp, C.POINTER(C.c_double),
                                            C.POINTER(C.c_uint)]),
    "azu_volume_refine_pose": (C.c_int, [vp, fp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, vp,
                                         C.c_float, C.c_int, fp, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    # tracker
    "azu_tracker_create": (C.c_int, [C.c_int, C.POINTER(TrackerParams), vp, C.POINTER(vp)]),
    "azu_tracker_destroy": (C.c_int, [vp]),
    "azu_tracker_set_params": (C.c_int, [vp, C.POINTER(TrackerParams)]),
    "azu_tracker_prepare_live": (C.c_int, [vp, vp, C.c_int, C.c_int]),
    "azu_tracker_track_prepared": (C.c_int, [vp, C.c_int, C.c_int, vp, vp, C.c_int, C.c_int, fp, fp,
                                             C.POINTER(IcpResult)]),
    "azu_tracker_track": (C.c_int, [vp, vp, C.c_int, C.c_int, vp, vp, C.c_int, C.c_int, fp, fp,
                                    C.POINTER(IcpResult)]),
    "azu_tracker_build_system": (C.c_int, [vp, C.c_int, vp, vp, C.c_int, C.c_int, fp, fp, fp, fp, fp,
                                           C.POINTER(C.c_int)]),
    "azu_tracker_track_many": (C.c_int, [vp, C.c_int, C.c_int, vp, vp, C.c_int, C.c_int, C.c_int, fp, fp,
                                         C.POINTER(TrackerParams), C.POINTER(IcpResult)]),
    "azu_tracker_load_live": (C.c_int, [vp, C.c_int, vp, vp, C.c_int, C.c_int]),
    "azu_icp_build_system_noalloc": (C.c_int, [vp, vp, C.c_int, C.c_int, vp, vp, C.c_int, C.c_int,
                                               C.POINTER(TrackerParams), fp, fp, vp, fp, fp, fp,
                                               C.POINTER(C.c_int)]),
    "azu_tracker_live_maps": (C.c_int, [vp, C.c_int, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]),
    "azu_testing_set_icp_wait": (C.c_int, [C.c_uint, C.c_uint]),
    # preprocessor
    "azu_preprocessor_create": (C.c_int, [C.c_int, C.c_int, vp, C.POINTER(vp)]),
    "azu_preprocessor_destroy": (C.c_int, [vp]),
    "azu_preprocessor_reset": (C.c_int, [vp]),
    "azu_preprocessor_reset_temporal": (C.c_int, [vp]),
    "azu_preprocessor_process": (C.c_int, [vp, vp, vp, C.c_float, C.c_float]),
    "azu_preprocessor_process_device": (C.c_int, [vp, vp, vp, C.c_float, C.c_float]),
    "azu_preprocessor_depth_meters": (vp, [vp]),
    "azu_preprocessor_rgb": (vp, [vp]),
    "azu_preprocessor_depth_raw": (vp, [vp]),
    "azu_preprocessor_luma": (vp, [vp]),
    # mesher
    "azu_mesher_create": (C.c_int, [C.c_int, vp, C.POINTER(vp)]),
    "azu_mesher_destroy": (C.c_int, [vp]),
    "azu_mesher_set_max_triangles": (C.c_int, [vp, C.c_int64]),
    "azu_mesher_extract": (C.c_int, [vp, vp, C.POINTER(MeshInfo)]),
    "azu_mesher_copy_out": (C.c_int, [vp, vp, vp, vp, vp]),
    "azu_mesher_device_buffers": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]),
    # pipeline
    "azu_pipeline_create": (C.c_int, [C.c_int, C.POINTER(PipelineParams), C.POINTER(vp)]),
    "azu_pipeline_destroy": (C.c_int, [vp]),
    "azu_pipeline_reset": (C.c_int, [vp]),
    "azu_pipeline_process_frame": (C.c_int, [vp, vp, vp, C.POINTER(FrameResult)]),
    "azu_pipeline_process_frame_device": (C.c_int, [vp, vp, vp, C.POINTER(FrameResult)]),
    "azu_pipeline_last_result": (C.c_int, [vp, C.POINTER(FrameResult)]),
    "azu_pipeline_volume": (vp, [vp]),
    "azu_pipeline_tracker": (vp, [vp]),
    "azu_pipeline_model_maps": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp)]),
    "azu_pipeline_stream": (vp, [vp]),
    "azu_pipeline_set_profiling": (C.c_int, [vp, C.c_int]),
    "azu_pipeline_stage_times": (C.c_int, [vp, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "azu_pipeline_uses_graph": (C.c_int, [vp]),
    # ingest
    "azu_recording_open": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
    "azu_recording_close": (None, [vp]),
    "azu_recording_frame_count": (C.c_int, [vp]),
    "azu_recording_frame_info": (C.c_int, [vp, C.c_int, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                           C.POINTER(C.c_int)]),
    "azu_recording_read": (C.c_int, [vp, C.c_int, vp, vp, C.POINTER(C.c_int)]),
    "azu_ingest_create": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.POINTER(vp)]),
    "azu_ingest_destroy": (C.c_int, [vp]),
    "azu_ingest_next": (C.c_int, [vp, C.POINTER(vp), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "azu_ingest_release": (C.c_int, [vp]),
    "azu_pipeline_process_frame_packed": (C.c_int, [vp, vp, C.POINTER(FrameResult)]),
    # export
    "azu_mesh_write_ply": (C.c_int, [C.c_char_p, C.c_int, vp, C.c_int64, vp, C.c_int64, vp, C.c_int64, vp,
                                     C.c_int64]),
    "azu_mesh_write_glb": (C.c_int, [C.c_char_p, vp, C.c_int64, vp, C.c_int64, vp, C.c_int64, vp, C.c_int64]),
    # batch
    "azu_batch_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(BatchScene), C.POINTER(vp)]),
    "azu_batch_destroy": (C.c_int, [vp]),
    "azu_batch_process": (C.c_int, [vp, C.POINTER(vp), C.c_int, C.POINTER(FrameResult)]),
    "azu_batch_autotune": (C.c_int, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "azu_batch_set_shapes": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int]),
    "azu_batch_get_shapes": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       C.POINTER(C.c_int)]),
    "azu_batch_volume": (vp, [vp, C.c_int]),
    "azu_batch_stream": (vp, [vp]),
    "azu_batch_uses_graph": (C.c_int, [vp]),
    "azu_batch_synchronize": (C.c_int, [vp]),
}


def header_symbols(header_path: str) -> list[str]:
    """Names of the functions declared in a C header of include/."""
    import re
    text = open(header_path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(azu_[a-z0-9_]+)\s*\(", text)))


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run azu_gb300.build.build() "
                               "(the CUDA backend has no fallback)")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


class AzuError(RuntimeError):
    def __init__(self, code, where):
        msg = load().azu_last_error().decode(errors="replace")
        super().__init__(f"{where} -> {code}: {msg}")
        self.code = code


def check(rc, where=""):
    if rc != AZU_OK:
        raise AzuError(rc, where)
    return rc
