// Setup::Setup() for the cross-check build of the reference (test
// infrastructure only).  The reference's potential factory names
// Setup::instance() inside its registration lambdas (include/factory_potential.h),
// so the linker needs the constructor, but the command-line and XML parameter
// reader that defines it (src/setup.cpp) is not compiled here: the harness
// builds every object directly.  Reaching it is an error.
#include "setup.h"

#include <stdexcept>

Setup::Setup() {
    throw std::logic_error("Setup is not part of the cross-check build; construct objects directly");
}
