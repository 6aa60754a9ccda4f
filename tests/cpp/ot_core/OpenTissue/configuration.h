// Test stand-in for OpenTissue's generated configuration.h (the drop-in
// C++ test builds against this minimal core where OpenTissue is absent).
#ifndef OPENTISSUE_CONFIGURATIOM_H
#define OPENTISSUE_CONFIGURATIOM_H
#include <string>
#endif
