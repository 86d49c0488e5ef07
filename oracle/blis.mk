# blis.mk -- compiles BLIS (flame/blis) straight from its C sources with gcc.
#
# This is a plain Makefile of this project, not the reference's build system:
# no configure step and no generated makefile fragments.  The two configuration
# headers BLIS's sources include (bli_config.h, bli_addon.h) are written into
# $(GEN) by oracle/ref_blis.py from the templates in the source tree
# (build/bli_config.h.in, build/bli_addon.h.in); every other header is read
# where it lies, without flattening, through one -I per source directory.
#
# The compile rules follow BLIS's own per-category flag sets (common.mk
# get-*-cflags-for and config/<cfg>/make_defs.mk):
#   framework (frame/)        COPT
#   framework noopt/          no optimisation (dlamch/slamch machine parameters)
#   config/<cfg>/*.c          COPT + -DBLIS_CNAME=<cfg>
#   kernels/<k>/              CKOPT CKVEC + -DBLIS_CNAME=<cfg>
#   ref_kernels/ (per cfg)    CROPT CRVEC -fopenmp-simd -DBLIS_IN_REF_KERNEL=1
#                             -include config/<cfg>/bli_kernel_defs_<cfg>.h,
#                             object names suffixed _<cfg>_ref
#   ref_kernels/bli_cntx_ref.c  COPT with the same reference-kernel macros
# Directories BLIS never compiles (build/gen-make-frags/ignore_list, plus the
# AMD framework tweaks, which BLIS compiles only on request) are skipped.
#
# Variables:
#   SRC      BLIS source root                         (required)
#   OUT      output directory                         (required)
#   GEN      directory holding bli_config.h, bli_addon.h  (default $(OUT)/gen)
#   CFG      sub-configuration (haswell, armsve, ...) (required)
#   KSETS    kernel sets of that sub-configuration    (required)
#   COPT CKOPT CKVEC CROPT CRVEC CPPROC   flag sets of CFG
#   SANDBOX  optional directory of a gemm sandbox (bli_sandbox.h + *.c),
#            compiled with the framework flags; bli_config.h must then define
#            BLIS_ENABLE_SANDBOX
#   SBOX_CFLAGS  extra flags for the sandbox sources
#   LIBEXTRA     extra linker arguments for libblis.so (a sandbox's own libraries)
#
# Targets: lib (libblis.so), testsuite (test_libblis.x objects), blastest
# (libf2c.a and the ?blat? objects).  Programs are linked by ref_blis.py so that
# the same objects serve the plain and the GPU-backed link orders.

SRC     ?=
OUT     ?=
GEN     ?= $(OUT)/gen
CFG     ?=
KSETS   ?=
COPT    ?= -O2
CKOPT   ?= -O3
CKVEC   ?=
CROPT   ?= $(CKOPT)
CRVEC   ?=
CPPROC  ?=
SANDBOX ?=
SBOX_CFLAGS ?=
LIBEXTRA ?=
CC      ?= gcc

ifeq ($(strip $(SRC)),)
$(error SRC (BLIS source root) is required)
endif
ifeq ($(strip $(OUT)),)
$(error OUT is required)
endif

CFG_UPPER := $(shell echo $(CFG) | tr a-z A-Z)
IGNORE    := attic broken old other temp tmp test p10_testsuite amd

# every .c under a directory, skipping the ignored directory names
prune      = $(foreach d,$(IGNORE),-name $(d) -o) -false
find_c     = $(shell find $(1) -type d \( $(prune) \) -prune -o -name '*.c' -print 2>/dev/null | sort)
find_dirs  = $(shell find $(1) -type d \( $(prune) \) -prune -o -type d -print 2>/dev/null | sort)

FRAME_SRC   := $(call find_c,$(SRC)/frame)
CONFIG_SRC  := $(wildcard $(SRC)/config/$(CFG)/*.c)
KERNEL_SRC  := $(foreach k,$(KSETS),$(call find_c,$(SRC)/kernels/$(k)))
REFK_SRC    := $(filter-out $(SRC)/ref_kernels/bli_cntx_ref.c,$(call find_c,$(SRC)/ref_kernels))
SBOX_SRC    := $(if $(SANDBOX),$(wildcard $(SANDBOX)/*.c))

INC_DIRS := $(GEN) $(call find_dirs,$(SRC)/frame) $(SRC)/config/$(CFG) \
            $(foreach k,$(KSETS),$(call find_dirs,$(SRC)/kernels/$(k))) \
            $(if $(SANDBOX),$(SANDBOX))
CINC     := $(addprefix -I,$(INC_DIRS))

CBASE    := -fPIC -std=c99 -D_POSIX_C_SOURCE=200112L -pthread $(CPPROC) -w $(CINC)
LIBDEF   := -DBLIS_IS_BUILDING_LIBRARY -fvisibility=hidden
CNAME    := -DBLIS_CNAME=$(CFG) -DBLIS_CNAME_UPPER=$(CFG_UPPER)
REFDEF   := $(CNAME) -DBLIS_IN_REF_KERNEL=1 -include $(SRC)/config/$(CFG)/bli_kernel_defs_$(CFG).h

O := $(OUT)/obj
obj_of = $(patsubst $(SRC)/%.c,$(O)/%.o,$(1))

FRAME_OBJ  := $(call obj_of,$(FRAME_SRC))
CONFIG_OBJ := $(call obj_of,$(CONFIG_SRC))
KERNEL_OBJ := $(call obj_of,$(KERNEL_SRC))
REFK_OBJ   := $(patsubst $(SRC)/ref_kernels/%.c,$(O)/ref_kernels/$(CFG)/%_$(CFG)_ref.o,$(REFK_SRC))
REFI_OBJ   := $(O)/ref_kernels/$(CFG)/bli_cntx_$(CFG)_ref.o
SBOX_OBJ   := $(patsubst $(SANDBOX)/%.c,$(O)/sandbox/%.o,$(SBOX_SRC))
LIB_OBJ    := $(FRAME_OBJ) $(CONFIG_OBJ) $(KERNEL_OBJ) $(REFK_OBJ) $(REFI_OBJ) $(SBOX_OBJ)

TS_SRC  := $(wildcard $(SRC)/testsuite/src/*.c)
TS_OBJ  := $(patsubst $(SRC)/testsuite/src/%.c,$(O)/testsuite/%.o,$(TS_SRC))
F2C_SRC := $(wildcard $(SRC)/blastest/f2c/*.c)
F2C_OBJ := $(patsubst $(SRC)/blastest/f2c/%.c,$(O)/blastest/f2c/%.o,$(F2C_SRC))
BT_SRC  := $(wildcard $(SRC)/blastest/src/*.c)
BT_OBJ  := $(patsubst $(SRC)/blastest/src/%.c,$(O)/blastest/src/%.o,$(BT_SRC))
BT_CFLAGS := -O2 -Wno-parentheses -I$(SRC)/blastest/f2c -DHAVE_BLIS_H

.PHONY: lib testsuite blastest all print-cflags
all: lib testsuite blastest
# the flags an application compiled against this tree's blis.h needs
print-cflags:
	@echo $(CBASE)
lib: $(OUT)/lib/libblis.so
testsuite: $(TS_OBJ)
blastest: $(OUT)/lib/libf2c.a $(BT_OBJ)

$(OUT)/lib/libblis.so: $(LIB_OBJ)
	@mkdir -p $(dir $@)
	$(CC) -shared -Wl,-soname,libblis.so -o $@ $(LIB_OBJ) $(LIBEXTRA) -lm -lpthread

$(OUT)/lib/libf2c.a: $(F2C_OBJ)
	@mkdir -p $(dir $@)
	rm -f $@ && ar cr $@ $(F2C_OBJ) && ranlib $@

# framework: the noopt directory (machine-parameter probes) is compiled without optimisation
$(O)/frame/base/noopt/%.o: $(SRC)/frame/base/noopt/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CBASE) $(LIBDEF) -c $< -o $@

$(O)/frame/%.o: $(SRC)/frame/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CBASE) $(COPT) $(LIBDEF) -c $< -o $@

$(O)/config/%.o: $(SRC)/config/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CBASE) $(COPT) $(CNAME) $(LIBDEF) -c $< -o $@

$(O)/kernels/%.o: $(SRC)/kernels/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CBASE) $(CKOPT) $(CKVEC) $(CNAME) $(LIBDEF) -c $< -o $@

$(O)/ref_kernels/$(CFG)/bli_cntx_$(CFG)_ref.o: $(SRC)/ref_kernels/bli_cntx_ref.c
	@mkdir -p $(dir $@)
	$(CC) $(CBASE) $(COPT) $(REFDEF) $(LIBDEF) -c $< -o $@

$(O)/ref_kernels/$(CFG)/%_$(CFG)_ref.o: $(SRC)/ref_kernels/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CBASE) $(CROPT) $(CRVEC) -fopenmp-simd $(REFDEF) $(LIBDEF) -c $< -o $@

$(O)/sandbox/%.o: $(SANDBOX)/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CBASE) $(COPT) $(LIBDEF) $(SBOX_CFLAGS) -c $< -o $@

$(O)/testsuite/%.o: $(SRC)/testsuite/src/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CBASE) -O2 -c $< -o $@

$(O)/blastest/f2c/%.o: $(SRC)/blastest/f2c/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CBASE) $(BT_CFLAGS) -c $< -o $@

$(O)/blastest/src/%.o: $(SRC)/blastest/src/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CBASE) $(BT_CFLAGS) -c $< -o $@
