/* openmps_gb300_defines.hpp - compile-time method switches of a C++ caller of
 * openmps_gb300.hpp, with the role of the reference's src/OpenMps/defines.hpp.
 *
 * The reference selects its method set with macros in defines.hpp (defines.hpp:9-56);
 * openmps_gb300.hpp reads the same macro names to form the runtime flags of
 * mps_params and the argument list of Environment.  This file defines the set the
 * reference ships (PRESSURE_GRADIENT_MIDPOINT, MPS_HS, MPS_HL, MPS_ECS, MPS_DS,
 * MPS_SPP).  It shares the reference file's include guard, so a caller that has
 * already included its own copy of the reference's defines.hpp keeps that choice and
 * this file adds nothing.  To change the method set, edit the list below as one edits
 * the reference's defines.hpp, or include the reference's own file first.
 */
#ifndef DEFINE_INCLUDED
#define DEFINE_INCLUDED

/* #define DIM3 */
#define PRESSURE_GRADIENT_MIDPOINT
/* #define PRESSURE_EXPLICIT */
#define MPS_HS
#define MPS_HL
#define MPS_ECS
/* #define MPS_GC */
#define MPS_DS
#define MPS_SPP

#endif
