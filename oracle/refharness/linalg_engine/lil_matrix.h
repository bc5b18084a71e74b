// Test infrastructure (oracle build only; never part of the product).
//
// The reference ships its LIL matrix as `include/linalg_engine/lil_matrix.h.j2`,
// a file with no template directives, i.e. plain C++.  Its build renames it to
// `lil_matrix.h`; this shim includes the reference file in place so that the
// reference's model headers (`qme_base.h:16`, `linalg_engine.h:18`) compile
// unchanged from their own sources.
#ifndef HEOMREF_SHIM_LIL_MATRIX_H
#define HEOMREF_SHIM_LIL_MATRIX_H
#include "utility.h"
#include "type.h"
#include "const.h"
#include "linalg_engine/lil_matrix.h.j2"
#endif
