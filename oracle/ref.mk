# Builds the reference's own serial CPU PLUTO for one problem configuration,
# straight from the reference sources with gcc (no setup.py, no generated
# makefile).  Test infrastructure only: the binary lands in
# oracle/_ref/<CFG>/ (git-ignored) and is used to generate and pin golden
# vectors for the oracle restatement.
#
#   make -f oracle/ref.mk CFG=blast2d [REF=<reference tree>]   (default $PLUTO_REF)
#
# Flags follow Config/Linux.gcc.defs of the reference (-O3 -std=c17, no
# -march, so no FMA contraction); the object list follows
# Src/Templates/makefile plus the module makefiles for HD, EOS/Ideal,
# Math_Tools and the RK2/PLM choices made by setup.py.

PLUTO_REF ?= /root/reference
REF     ?= $(PLUTO_REF)
CFG     ?= blast2d
HERE    := $(dir $(abspath $(lastword $(MAKEFILE_LIST))))
CFGDIR  := $(HERE)ref_cfg/$(CFG)
OUT     := $(HERE)_ref/$(CFG)
SRC     := $(REF)/Src

CC      := gcc
CFLAGS  := -O3 -std=c17 -w
LDFLAGS := -lm

SRCDIRS := $(SRC) $(SRC)/HD $(SRC)/MHD $(SRC)/EOS/Ideal $(SRC)/States \
           $(SRC)/Time_Stepping $(SRC)/Math_Tools
INCS    := -I$(CFGDIR) -I$(SRC) -I$(SRC)/HD -I$(SRC)/EOS/Ideal \
           -I$(SRC)/States -I$(SRC)/Math_Tools

OBJ := adv_flux.o arrays.o array_reconstruct.o boundary.o check_states.o \
       cmd_line_opt.o debug_tools.o entropy_switch.o failsafe.o \
       flag_shock.o flatten.o fluid_interface_boundary.o get_nghost.o \
       init.o int_bound_reset.o input_data.o mappers3D.o mean_mol_weight.o \
       parse_file.o plm_coeffs.o rbox.o reconstruct.o rotate.o \
       set_indexes.o set_geometry.o set_output.o tools.o var_names.o \
       bin_io.o colortable.o initialize.o jet_domain.o main.o output_log.o \
       restart.o ring_average.o runtime_setup.o set_image.o show_config.o \
       set_grid.o startup.o split_source.o userdef_output.o write_data.o \
       write_tab.o write_img.o write_vtk.o write_vtk_proc.o \
       math_interp.o math_lu_decomp.o math_qr_decomp.o math_misc.o \
       math_ode.o math_quadrature.o math_random.o math_root_finders.o \
       math_table2D.o \
       advection_solver.o ausm.o eigenv.o fluxes.o mappers.o mappers_loc.o \
       hll_speed.o hll.o hllc.o set_solver.o tvdlf.o two_shock.o roe.o \
       prim_eqn.o rhs.o rhs_source.o eos.o plm_states.o rk_step.o \
       update_stage.o

# Extra modules for the line-driven wind configurations.
ifneq ($(wildcard $(CFGDIR)/WIND),)
SRCDIRS += $(SRC)/Cooling/BLONDIN $(SRC)/LineDriven
INCS    += -I$(SRC)/Cooling/BLONDIN -I$(SRC)/LineDriven
OBJ     += cooling.o line_connect.o
endif

# The wind with the ODE cooling path (COOLING TABULATED): the generic
# integrators (Src/Cooling/cooling_ode_solver.c, Tabulated/) with the
# production problem's own CoolingSource and Radiat (BLONDIN rates as the
# right-hand side), compiled where they lie in Test_Problems.
ifneq ($(wildcard $(CFGDIR)/WIND_ODE),)
CVIDL   := $(REF)/Test_Problems/LineDrivenWind/cv_idl
SRCDIRS += $(SRC)/LineDriven $(SRC)/Cooling $(SRC)/Cooling/Tabulated
INCS    += -I$(SRC)/LineDriven -I$(SRC)/Cooling
OBJ     += line_connect.o cooling_ode_solver.o jacobian.o maxrate.o cv_radiat.o cv_cooling_source.o
endif

# The production disk-wind problem itself (marker CVIDL): its own
# definitions.h and init.c (UserDefBoundary, BodyForceVector, Init), and
# the rest of its directory, compiled where they lie; the configuration
# directory only holds pluto.ini.
DEFS    := $(CFGDIR)/definitions.h
PROBDIR := $(CFGDIR)
ifneq ($(wildcard $(CFGDIR)/CVIDL),)
PROBDIR := $(REF)/Test_Problems/LineDrivenWind/cv_idl
DEFS    := $(PROBDIR)/definitions.h
INCS    := -I$(PROBDIR) $(filter-out -I$(CFGDIR),$(INCS))
endif

# The problem directory comes first so that its init.c (and any file it
# overrides) wins, as with PLUTO's own VPATH.
VPATH := $(PROBDIR) $(SRCDIRS)

OBJS := $(addprefix $(OUT)/,$(OBJ))

all: $(OUT)/pluto $(OUT)/pluto.ini

$(OUT)/pluto: $(OBJS)
	$(CC) $(OBJS) $(LDFLAGS) -o $@

# The reference's own main loop with the GB300 path dropped in: PLUTO's
# objects without AdvanceStep (rk_step.o) and SplitSource (split_source.o),
# plus the shim that calls libps_gb300.so through include/ps_gb300.h.
#   make -f oracle/ref.mk CFG=<cfg> shim   -> oracle/_ref/<cfg>/pluto_gb300
PKG      := $(abspath $(HERE)../pluto-sirocco_gb300)
SHIM_OBJS := $(filter-out $(OUT)/rk_step.o $(OUT)/split_source.o,$(OBJS)) $(OUT)/ps_pluto_shim.o

shim: $(OUT)/pluto_gb300 $(OUT)/pluto.ini

$(OUT)/ps_pluto_shim.o: $(PKG)/shim/ps_pluto_shim.c $(HERE)../include/ps_gb300.h \
                        $(DEFS) | $(OUT)
	$(CC) $(CFLAGS) $(INCS) -I$(HERE)../include -include string.h -c $< -o $@

$(OUT)/pluto_gb300: $(SHIM_OBJS) $(PKG)/libps_gb300.so
	$(CC) $(SHIM_OBJS) -L$(PKG) -lps_gb300 -Wl,-rpath,$(PKG) $(LDFLAGS) -o $@

$(OUT)/pluto.ini: $(CFGDIR)/pluto.ini
	cp $< $@

$(OUT)/%.o: %.c $(DEFS) | $(OUT)
	$(CC) $(CFLAGS) $(INCS) -c $< -o $@

$(OUT)/cv_radiat.o: $(CVIDL)/radiat.c $(DEFS) | $(OUT)
	$(CC) $(CFLAGS) $(INCS) -c $< -o $@

$(OUT)/cv_cooling_source.o: $(CVIDL)/cooling_source.c $(DEFS) | $(OUT)
	$(CC) $(CFLAGS) $(INCS) -c $< -o $@

$(OUT):
	mkdir -p $@

.PHONY: all shim
