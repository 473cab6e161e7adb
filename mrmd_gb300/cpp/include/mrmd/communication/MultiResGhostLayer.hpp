// Drop-in communication::MultiResGhostLayer
// (communication/MultiResGhostLayer.hpp:29-61): declared beside GhostLayer,
// from which it derives.
#pragma once

#include "GhostLayer.hpp"
