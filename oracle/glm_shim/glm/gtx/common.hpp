// Part of the glm stand-in used only to compile the reference into the checker
// library; the compiled sources need nothing from this header.
#pragma once
#include "../glm.hpp"
