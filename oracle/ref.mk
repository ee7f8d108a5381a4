# Builds the reference LightsprintCore library from its own sources, where
# they lie, into oracle/_ref/ (git-ignored).  Test infrastructure only: the
# result is the parity oracle and the CPU baseline measured in this container;
# nothing in the product links it.
#
#   make -f oracle/ref.mk -j8 REF=/root/reference
#
# Flags follow the reference's own linux configuration (src/configs/
# linux.common, linux.release: -std=c++17 -O2 -fopenmp, RR_BUILD) with three
# additions that let it build without Boost: our compat headers under
# oracle/compat, -D_strdup=strdup and two forced includes.
REF      ?= /root/reference
CORE     := $(REF)/src/LightsprintCore
OUT      := oracle/_ref
CXX      ?= g++
CXXFLAGS := -std=c++17 -O2 -fopenmp -DNDEBUG -DRR_BUILD -D_strdup=strdup \
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
# workloads' binary inputs and write binary outputs.
DRIVERS := $(OUT)/ref_collide $(OUT)/ref_filter $(OUT)/ref_enumerate $(OUT)/ref_gather

all: $(OUT)/libLightsprintCore.a $(DRIVERS)

$(OUT)/obj/%.o: $(CORE)/%.cpp
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/libLightsprintCore.a: $(OBJS)
	rm -f $@
	ar rcs $@ $(OBJS)

$(OUT)/%: oracle/%.cpp $(OUT)/libLightsprintCore.a
	$(CXX) $(CXXFLAGS) $< -o $@ $(OUT)/libLightsprintCore.a -lgomp -lpthread

.PHONY: all
