// Stand-in for the AMGCL header of the same name: AMGCL cannot be built without Boost,
// so every AMGCL include of the reference resolves to the facade below.
#pragma once
#include "../facade.hpp"
