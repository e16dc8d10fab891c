# ORACLE -- test infrastructure only.
#
# Builds oracle/_ref/libmpart_ref.so from the reference's own sources, where
# they lie (REF, read-only), compiled unchanged against the serial Kokkos,
# minimal Eigen and save-side cereal stand-ins in oracle/ref_shim/ (with the
# reference's archive support on, MPART_HAS_CEREAL), plus oracle/ref_driver.cpp
# (C entry points).  Outputs go to oracle/_ref/ only.  The reference's own
# build system is not used: these are the few sources of the monotone-
# component path (map base classes, TriangularMap, the component factory
# registrations for ProbabilistHermite / HermiteFunctions with every
# quadrature kind, the multi-index sets).  Strict IEEE evaluation order
# (-ffp-contract=off), as the oracle's parity build, so that the two are
# compared like for like; asserts stay on, as in the reference's release
# flags (CMakeLists.txt:49, "-O3" without -DNDEBUG).
#
#   make -f oracle/ref.mk REF=<path of the reference checkout>
REF ?= /root/reference
HERE := $(dir $(lastword $(MAKEFILE_LIST)))
OUT := $(HERE)_ref
CXX ?= g++
CXXFLAGS := -O2 -std=c++17 -fPIC -ffp-contract=off -fno-fast-math -w -DMPART_HAS_CEREAL -I$(HERE)ref_shim -I$(REF)

SRCS := src/ParameterizedFunctionBase.cpp src/ConditionalMapBase.cpp src/TriangularMap.cpp \
        src/MapFactoryImpl4.cpp src/MapFactoryImpl5.cpp src/MapFactoryImpl6.cpp \
        src/MapFactoryImpl7.cpp src/MapFactoryImpl8.cpp src/MapFactoryImpl9.cpp \
        src/MultiIndices/FixedMultiIndexSet.cpp src/MultiIndices/MultiIndex.cpp \
        src/MultiIndices/MultiIndexSet.cpp src/MultiIndices/MultiIndexLimiter.cpp \
        src/MultiIndices/MultiIndexNeighborhood.cpp src/Utilities/Miscellaneous.cpp
OBJS := $(addprefix $(OUT)/obj/,$(notdir $(SRCS:.cpp=.o))) $(OUT)/obj/ref_driver.o
SHIMS := $(HERE)ref_shim/Kokkos_Core.hpp $(HERE)ref_shim/Eigen/Core $(HERE)ref_shim/cereal/cereal.hpp

all: $(OUT)/libmpart_ref.so

$(OUT)/libmpart_ref.so: $(OBJS)
	$(CXX) -shared -Wl,--no-undefined -o $@ $^

$(OUT)/obj/ref_driver.o: $(HERE)ref_driver.cpp $(SHIMS)
	@mkdir -p $(OUT)/obj
	$(CXX) $(CXXFLAGS) -c $< -o $@

define ref_rule
$(OUT)/obj/$(notdir $(1:.cpp=.o)): $(REF)/$(1) $(SHIMS)
	@mkdir -p $(OUT)/obj
	$(CXX) $(CXXFLAGS) -c $$< -o $$@
endef
$(foreach s,$(SRCS),$(eval $(call ref_rule,$(s))))

clean:
	rm -rf $(OUT)

.PHONY: all clean
