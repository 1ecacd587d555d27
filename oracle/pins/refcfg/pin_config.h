// Hand-written build configuration of the reference sources compiled by
// oracle/pins/ecsim_pin.cpp, in place of what the reference's configuration
// script would generate for its fast-wave test input
// (input/test/fast-wave.input): electromagnetic ECSIM field solver with the
// corner-based magnetic field, normalised units, one global time step,
// species-dependent global particle weights with individual weight
// corrections.  Mover::Boris takes its force through the reference's hook
// _PIC_PARTICLE_MOVER__BORIS_SPLIT_ACCELERATION_ (picGlobal.dfn:125), which
// a model overrides with its own field source; here it is the harness's
// pin_boris_split_acceleration (the Lorentz part of
// BorisSplitAcceleration_default on the harness's corner fields).  pic.h fixes PIC::nTotalSpecies at 1 (the configuration script
// rewrites that line), so the harness runs one species at a time.
//
// src/pic/pic.h includes src/pic/picGlobal.dfn (the defaults) and then the
// coupler header FluidPicInterface.h, whose stand-in includes this file, so
// these definitions replace the defaults.
#pragma once
#undef _PIC_FIELD_SOLVER_MODE_
#define _PIC_FIELD_SOLVER_MODE_ _PIC_FIELD_SOLVER_MODE__ELECTROMAGNETIC__ECSIM_
#undef _PIC_FIELD_SOLVER_B_MODE_
#ifdef PIN_B_CENTER
// the reference's default magnetic-field placement (picGlobal.dfn), with the
// cell-centred linear interpolation its ECSIM test inputs select
// (cell_centered_linear_interpolation_mode=amps, input/test/fast-wave.input:90,
// which ampsConfig.pl:2927-2931 turns into these two macros)
#define _PIC_FIELD_SOLVER_B_MODE_ _PIC_FIELD_SOLVER_B_CENTER_BASED_
#undef _PIC_COUPLER__INTERPOLATION_MODE_
#define _PIC_COUPLER__INTERPOLATION_MODE_ _PIC_COUPLER__INTERPOLATION_MODE__CELL_CENTERED_LINEAR_
#undef _PIC_CELL_CENTERED_LINEAR_INTERPOLATION_ROUTINE_
#define _PIC_CELL_CENTERED_LINEAR_INTERPOLATION_ROUTINE_ _PIC_CELL_CENTERED_LINEAR_INTERPOLATION_ROUTINE__AMPS_
#else
#define _PIC_FIELD_SOLVER_B_MODE_ _PIC_FIELD_SOLVER_B_CORNER_BASED_
#endif
#undef _PIC_FIELD_SOLVER_INPUT_UNIT_
#define _PIC_FIELD_SOLVER_INPUT_UNIT_ _PIC_FIELD_SOLVER_INPUT_UNIT_NORM_
#undef _SIMULATION_TIME_STEP_MODE_
#define _SIMULATION_TIME_STEP_MODE_ _SINGLE_GLOBAL_TIME_STEP_
#define _TOTAL_SPECIES_NUMBER_ 1
#undef _PIC_PARTICLE_MOVER__BORIS_SPLIT_ACCELERATION_
#define _PIC_PARTICLE_MOVER__BORIS_SPLIT_ACCELERATION_(accl, rotation, spec, ptr, x, v, startNode) \
  pin_boris_split_acceleration(accl, rotation, spec, ptr, x, v, startNode);
void pin_boris_split_acceleration(double* accl, double* rotation, int spec, long int ptr, double* x,
                                  double* v, void* startNode);
