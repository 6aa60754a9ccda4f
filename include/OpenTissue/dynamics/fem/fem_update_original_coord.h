#ifndef OPENTISSUE_DYNAMICS_FEM_FEM_UPDATE_ORIGINAL_COORD_H
#define OPENTISSUE_DYNAMICS_FEM_FEM_UPDATE_ORIGINAL_COORD_H
//
// Drop-in GB300 implementation of OpenTissue/dynamics/fem.
// fem::update_original_coord (reference: fem_update_original_coord.h:28-33):
// m_model_coord = m_coord for every node in the range.  The host node is the
// authoritative copy; fem::simulate sends m_model_coord to the device every
// step, so the next step uses the new rest positions (the element stiffness
// from fem::init is kept, as in the reference).
//
#include <OpenTissue/configuration.h>

namespace OpenTissue {
namespace fem {

template <typename node_iterator>
inline void update_original_coord(node_iterator const& begin, node_iterator const& end) {
  for (node_iterator n = begin; n != end; ++n) n->m_model_coord = n->m_coord;
}

}  // namespace fem
}  // namespace OpenTissue

#endif
