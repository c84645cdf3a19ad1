// TEST INFRASTRUCTURE -- stand-in header (see MOF.hpp).
#pragma once
#include "MOF.hpp"
