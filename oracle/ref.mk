# Builds the reference NCrystal library (libNCrystal.so) straight from its
# C++ sources, without running the reference's own build system.
#
# Test infrastructure only: the library is the oracle's oracle.  It is used to
#   * pin the C restatement in oracle/ against the real implementation,
#   * export material bundles (ncrystal_gb300/bundle/ncgb_export.cc),
#   * generate the committed golden fixtures under tests/golden/.
# Outputs go to oracle/_ref/ only (git-ignored).  The reference sources are read
# where they lie; nothing is copied into the repository.
#
#   make -f oracle/ref.mk -j8 REFDIR=<NCrystal source tree>
#
# The only configure-time file of the reference is include/NCrystal/ncapi.h,
# made from ncapi.h.in by replacing the @NCRYSTAL_HOOK_FOR_ADDING_DEFINES@
# comment hook with five version #defines (the reference's Python layer checks
# the version).  That substitution is done here with sed into oracle/_ref/gen/.  Data files are read from the
# reference's data/ directory (NCRYSTAL_DATADIR) instead of being embedded.
# One source (utils/NCCFileUtils.cc) relies on <stdexcept> arriving transitively,
# which this libstdc++ does not do, hence the forced include.

ifndef REFDIR
$(error REFDIR must name the NCrystal source tree)
endif
OUT    ?= oracle/_ref
CORE   := $(REFDIR)/ncrystal_core
CXX    ?= g++
SRCS   := $(shell find $(CORE)/src -name '*.cc' | sort)
OBJS   := $(patsubst $(CORE)/src/%.cc,$(OUT)/obj/%.o,$(SRCS))
# Release-like flags.  -ffp-contract=off keeps the arithmetic identical on
# x86-64 and aarch64 (gcc contracts a*b+c into fma on aarch64 by default).
CXXFLAGS := -std=c++17 -O2 -DNDEBUG -fPIC -ffp-contract=off -include stdexcept \
            -DNCRYSTAL_DATADIR=$(REFDIR)/data -DNCRYSTAL_NO_CMATH_CONSTANTS \
            -I$(OUT)/gen -I$(CORE)/include -I$(CORE)/src

all: $(OUT)/libNCrystal.so

VERSION := $(shell cat $(REFDIR)/VERSION)
VMAJ := $(word 1,$(subst ., ,$(VERSION)))
VMIN := $(word 2,$(subst ., ,$(VERSION)))
VPAT := $(word 3,$(subst ., ,$(VERSION)))
VINT := $(shell echo $$(( $(VMAJ)*1000000 + $(VMIN)*1000 + $(VPAT) )))

$(OUT)/gen/NCrystal/ncapi.h: $(CORE)/include/NCrystal/ncapi.h.in
	@mkdir -p $(dir $@)
	sed 's|@NCRYSTAL_HOOK_FOR_ADDING_DEFINES@|*/\n#define NCRYSTAL_VERSION_MAJOR $(VMAJ)\n#define NCRYSTAL_VERSION_MINOR $(VMIN)\n#define NCRYSTAL_VERSION_PATCH $(VPAT)\n#define NCRYSTAL_VERSION $(VINT)\n#define NCRYSTAL_VERSION_STR "$(VERSION)"\n/*|' $< > $@

$(OUT)/obj/%.o: $(CORE)/src/%.cc $(OUT)/gen/NCrystal/ncapi.h
	@mkdir -p $(dir $@)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/libNCrystal.so: $(OBJS)
	$(CXX) -shared -o $@ $(OBJS) -lpthread -ldl -lm

.PHONY: all
