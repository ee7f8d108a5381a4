# Builds the reference LightsprintCore library from its own sources into
# oracle/_ref/ (git-ignored).  Test infrastructure only: the result is the
# parity oracle, the reference side of the plugin tests and the CPU baseline;
# nothing in the product links it.
#
#   make -f oracle/ref.mk stage REF_SRC=/root/reference   # where the reference lies
#   make -f oracle/ref.mk -j8                             # build from the staged copy
#
# `stage` copies the sources this build reads (src/LightsprintCore and the
# Lightsprint and embree3 headers) unchanged into oracle/_ref/src, which is
# git-ignored but travels with the working tree to machines that have no
# reference checkout (the GPU host), so that the same recipe builds the
# library there.  cp -p keeps the files' times, so restaging leaves make's
# view of what is up to date unchanged.
#
# Flags follow the reference's own linux configuration (src/configs/
# linux.common, linux.release: -std=c++17 -O2 -fopenmp, RR_BUILD) with these
# additions: our compat headers under oracle/compat (no Boost),
# -D_strdup=strdup, two forced includes, and -fsigned-char -ffp-contract=off
# so that an aarch64 build computes what the x86-64 build does (GCC contracts
# a*b+c into fused multiply-adds by default for C++ where the target has
# them, as aarch64 does; x86-64 without -mfma has none).
REF_SRC  ?= /root/reference
REF      := oracle/_ref/src
CORE     := $(REF)/src/LightsprintCore
OUT      := oracle/_ref
CXX      ?= g++
CXXFLAGS := -std=c++17 -O2 -fopenmp -DNDEBUG -DRR_BUILD -D_strdup=strdup -fsigned-char -ffp-contract=off \
            -include string -include climits -fPIC -w \
            -I$(REF)/include -I$(CORE) -Ioracle/compat

SOURCES := \
  RRBuffer/RRBuffer.cpp RRBuffer/RRBufferBlend.cpp RRBuffer/RRBufferInMemory.cpp \
  RRReporter/RRReporter.cpp RRReporter/RRReporterFile.cpp \
  RRReporter/RRReporterOutputDebugString.cpp RRReporter/RRReporterPrintf.cpp \
  RRReporter/RRReporterWindow.cpp RRReporter/RRReportInterval.cpp \
  RRCollider/bsp.cpp RRCollider/EmbreeCollider.cpp RRCollider/fpcube.cpp \
  RRCollider/geometry.cpp RRCollider/IntersectBspCompact.cpp \
  RRCollider/IntersectBspFast.cpp RRCollider/IntersectLinear.cpp \
  RRCollider/IntersectVerification.cpp RRCollider/pcube.cpp \
  RRCollider/RRCollider.cpp RRCollider/RRColliderMulti.cpp RRCollider/RRRay.cpp \
  RRHash/sha1.cpp RRHash/RRHash.cpp \
  RRMesh/RRMesh.cpp RRMesh/RRMeshAccelerated.cpp RRMesh/RRMeshArrays.cpp \
  RRMesh/RRMeshLessVertices.cpp \
  RRObject/RRMaterial.cpp RRObject/RRObject.cpp RRObject/RRObjects.cpp \
  RRPackedSolver/PackedSolverFileBuild.cpp RRPackedSolver/RRPackedSolver.cpp \
  RRSolver/environmentMap.cpp RRSolver/gather.cpp RRSolver/lightmap.cpp \
  RRSolver/RRSolver.cpp RRSolver/vertexBuffer.cpp \
  RRStaticSolver/geometry_v.cpp RRStaticSolver/interpol.cpp \
  RRStaticSolver/pathtracer.cpp RRStaticSolver/rrcore.cpp \
  RRStaticSolver/RRStaticSolver.cpp \
  squish/alpha.cpp squish/clusterfit.cpp squish/colourblock.cpp \
  squish/colourfit.cpp squish/colourset.cpp squish/maths.cpp \
  squish/rangefit.cpp squish/singlecolourfit.cpp squish/squish.cpp \
  Preferences.cpp RRCamera.cpp RRColorSpace.cpp RRFileLocator.cpp RRLight.cpp \
  RRLightField.cpp RRMath.cpp RRMemory.cpp RRObjectIllumination.cpp \
  RRScene.cpp RRTime.cpp Unwrapper.cpp

OBJS := $(addprefix $(OUT)/obj/,$(SOURCES:.cpp=.o))

# Drivers (our code) that run the reference collider and gather on the
# workloads' binary inputs and write binary outputs, and the shared library
# through which the benchmark times the reference collider in-process.
DRIVERS := $(OUT)/ref_collide $(OUT)/ref_filter $(OUT)/ref_enumerate $(OUT)/ref_gather

all: $(OUT)/libLightsprintCore.a $(DRIVERS) $(OUT)/libref_bench.so

stage:
	@test -d $(REF_SRC)/src/LightsprintCore || { echo "no reference sources under $(REF_SRC)"; exit 1; }
	@mkdir -p $(REF)/src $(REF)/include
	@cp -rp $(REF_SRC)/src/LightsprintCore $(REF)/src/
	@cp -rp $(REF_SRC)/include/Lightsprint $(REF_SRC)/include/embree3 $(REF)/include/

$(OUT)/obj/%.o: $(CORE)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/libLightsprintCore.a: $(OBJS)
	rm -f $@
	ar rcs $@ $(OBJS)

$(OUT)/libref_bench.so: oracle/ref_bench.cpp $(OUT)/libLightsprintCore.a
	$(CXX) $(CXXFLAGS) -shared $< -o $@ $(OUT)/libLightsprintCore.a -lgomp -lpthread

$(OUT)/%: oracle/%.cpp $(OUT)/libLightsprintCore.a
	$(CXX) $(CXXFLAGS) $< -o $@ $(OUT)/libLightsprintCore.a -lgomp -lpthread

.PHONY: all stage
