#ifndef OPENTISSUE_DYNAMICS_FEM_FEM_H
#define OPENTISSUE_DYNAMICS_FEM_FEM_H
//
// Drop-in GB300 implementation of OpenTissue/dynamics/fem (reference umbrella:
// fem.h:12-16).  Put this repository's include/ directory before the
// OpenTissue source root on the include path and link libotfem_gpu.so; the
// rest of OpenTissue (math types, t4mesh) is used unchanged.
//
#include <OpenTissue/configuration.h>

#include <OpenTissue/dynamics/fem/fem_mesh.h>
#include <OpenTissue/dynamics/fem/fem_init.h>
#include <OpenTissue/dynamics/fem/fem_update_original_coord.h>
#include <OpenTissue/dynamics/fem/fem_export_k.h>
#include <OpenTissue/dynamics/fem/fem_simulate.h>
#include <OpenTissue/dynamics/fem/fem_detail.h>

#endif
