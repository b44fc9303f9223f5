// Empty stand-in (see ptree.hpp).
#pragma once
#include "ptree.hpp"
