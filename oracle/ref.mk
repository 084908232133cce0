# Oracle (test infrastructure only): builds the REFERENCE's own hot-path sources,
# unmodified from where they lie, against the project's Eigen-API shim
# (eigen_shim/; Eigen is not installed here), with the C entry points of
# ref_capi.cpp, into oracle/_ref/libazu_ref.so. Outputs go to oracle/_ref/ only.
#
#   make -f ref.mk REF=<path of the reference checkout>
#
# Flags follow the reference's test build: -O2 -fopenmp, no fused multiply-add
# (-ffp-contract=off), and the pipeline test seam the reference's own contract
# tests build with (-DAZU_PIPELINE_TEST_SEAM). No Qt, libfreenect or GPU code is
# compiled: none of these sources needs them.
REF      ?= /root/reference
CXX      ?= g++
CXXFLAGS ?= -O2 -std=c++17 -fPIC -fopenmp -ffp-contract=off -fno-fast-math -w -DAZU_PIPELINE_TEST_SEAM
INC      := -I eigen_shim -I $(REF)/include -I $(REF)/src -I $(REF)/third_party/tinygltf -I .
SRC      := $(REF)/src/tsdf/TSDFVolume.cpp $(REF)/src/tracking/ICPTracker.cpp $(REF)/src/sensor/FrameData.cpp \
            $(REF)/src/meshing/MarchingCubes.cpp $(REF)/src/sensor/SignalConditioner_omp.cpp \
            $(REF)/src/sensor/SuperResolution.cpp $(REF)/src/sensor/KinectSensor.cpp \
            $(REF)/src/export/PLYExporter.cpp $(REF)/src/export/GLBExporter.cpp \
            $(REF)/src/utils/Logger.cpp $(REF)/src/utils/Timer.cpp
OBJ      := $(patsubst $(REF)/src/%.cpp,_ref/obj/%.o,$(SRC)) _ref/obj/ref_capi.o
OUT      := _ref/libazu_ref.so
SHIM     := $(wildcard eigen_shim/Eigen/* eigen_shim/Eigen/src/*) orc_linalg.h orc_math.h

all: $(OUT)

_ref/obj/%.o: $(REF)/src/%.cpp $(SHIM)
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@

_ref/obj/ref_capi.o: ref_capi.cpp orc_api.h $(SHIM)
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@

$(OUT): $(OBJ)
	$(CXX) $(CXXFLAGS) -shared -o $@ $(OBJ)

# The reference's own contract tests of the path (its tests/*.cpp, each a
# program that exits 0 when every check passes), linked against the same
# objects: they pin this build, shim included, to the reference's hand-derived
# expectations.
CONTRACTS := tsdf_integration_race_contract tsdf_integration_min_depth_contract fusion_bias_contract \
             tsdf_raycast_contract tsdf_subvoxel_thin_feature_contract raycast_accuracy_contract \
             tsdf_reset_contract coordinate_rounding_contract icp_weighting_contract icp_numeric_policy_contract \
             icp_refpose_contract icp_lowres_model_contract tracking_policy_contract depth_consistency_contract \
             marching_cubes_table_contract mesh_welding_contract \
             marching_cubes_winding_contract marching_cubes_frontier_contract mesh_truncation_progress_contract \
             marching_cubes_sphere_contract mesh_color_invariant_contract mesh_validation_contract \
             depth_domain_contract depth_ema_determinism_contract cas_border_contract ply_writer_contract \
             glb_writer_contract glb_linear_color_contract kinect_pairing_contract
CONTRACT_BIN := $(addprefix _ref/contracts/,$(CONTRACTS))
REF_OBJ := $(filter-out _ref/obj/ref_capi.o,$(OBJ))

contracts: $(CONTRACT_BIN)

_ref/contracts/%: $(REF)/tests/%.cpp $(REF_OBJ)
	@mkdir -p _ref/contracts
	$(CXX) $(CXXFLAGS) $(INC) -I $(REF)/tests -o $@ $< $(REF_OBJ)

clean:
	rm -rf _ref

.PHONY: all clean contracts
