# ref.mk — builds the reference engine (SlothDB) from its own sources with
# plain g++/gcc, and links the parity harness (oracle/ref_harness.cpp) to it.
#
# TEST INFRASTRUCTURE ONLY.  The library and harness it makes are the
# checker that pins the oracle to the reference itself; nothing in the
# product links or loads them.
#
# This does not run the reference's own build system: it compiles the
# source files its build globs (every .cpp under src/, the vendored
# decompression-only zstd, fastpforlib's bitpacking.cpp and snappy), with
# the definitions that build sets for them, into objects under
# oracle/_ref/obj.  No generated sources are involved (the vendored snappy
# ships its configured headers).  Outputs go only to oracle/_ref/.
#
#   make -f oracle/ref.mk REF=/root/reference -j8
#
# REF defaults to the reference checkout in this container.

REF ?= /root/reference
OUT ?= $(dir $(abspath $(lastword $(MAKEFILE_LIST))))_ref
OBJ := $(OUT)/obj
HERE := $(dir $(abspath $(lastword $(MAKEFILE_LIST))))

CXX ?= g++
CC ?= gcc
ARCHFLAGS :=
ifeq ($(shell uname -m),x86_64)
  # the reference's own build adds AVX2 code generation on x86-64
  ARCHFLAGS := -mavx2
endif

INC := -I$(REF)/include -I$(REF)/third_party/zstd/lib -I$(REF)/third_party/fastpforlib -I$(REF)/third_party/snappy
CXXFLAGS := -std=c++20 -O2 -fPIC -w $(ARCHFLAGS) $(INC)
CFLAGS := -O2 -fPIC -w $(INC)

SRC_CPP := $(shell find $(REF)/src -name '*.cpp' -not -path '*/tools/*' | sort)
SRC_C := $(REF)/src/storage/miniz.c
ZSTD := $(addprefix $(REF)/third_party/zstd/lib/, common/debug.c common/entropy_common.c common/error_private.c \
          common/fse_decompress.c common/pool.c common/threading.c common/xxhash.c common/zstd_common.c \
          decompress/huf_decompress.c decompress/zstd_ddict.c decompress/zstd_decompress.c \
          decompress/zstd_decompress_block.c)
FASTPFOR := $(REF)/third_party/fastpforlib/bitpacking.cpp
SNAPPY := $(addprefix $(REF)/third_party/snappy/, snappy.cc snappy-sinksource.cc snappy-stubs-internal.cc snappy-c.cc)

obj_of = $(OBJ)/$(subst /,_,$(patsubst $(REF)/%,%,$(1))).o
OBJS := $(foreach s,$(SRC_CPP) $(SRC_C) $(ZSTD) $(FASTPFOR) $(SNAPPY),$(call obj_of,$(s)))

all: $(OUT)/libslothdb_ref.a $(OUT)/ref_harness

define cxx_rule
$(call obj_of,$(1)): $(1)
	@mkdir -p $(OBJ)
	$(CXX) $(CXXFLAGS) -c $$< -o $$@
endef
define c_rule
$(call obj_of,$(1)): $(1)
	@mkdir -p $(OBJ)
	$(CC) $(CFLAGS) $(2) -c $$< -o $$@
endef

$(foreach s,$(SRC_CPP) $(FASTPFOR) $(SNAPPY),$(eval $(call cxx_rule,$(s))))
$(foreach s,$(SRC_C),$(eval $(call c_rule,$(s),)))
$(foreach s,$(ZSTD),$(eval $(call c_rule,$(s),-DZSTD_DISABLE_ASM=1 -DZSTD_MULTITHREAD=0)))

$(OUT)/libslothdb_ref.a: $(OBJS)
	rm -f $@
	ar rcs $@ $^

$(OUT)/ref_harness: $(HERE)ref_harness.cpp $(OUT)/libslothdb_ref.a
	$(CXX) -std=c++20 -O2 -I$(REF)/include $< -o $@ $(OUT)/libslothdb_ref.a -lpthread

.PHONY: all
