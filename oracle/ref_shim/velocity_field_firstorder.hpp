// TEST INFRASTRUCTURE -- stand-in header (see velocity_field.hpp).
#pragma once
#include "velocity_field.hpp"
