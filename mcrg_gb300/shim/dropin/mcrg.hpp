// mcrg.hpp -- drop-in for kim-jane/MCRG src/mcrg.hpp:
// MonteCarloRenormalizationGroup over the GPU (declared with Lattice in
// ../mcrg_classes.hpp).
#pragma once
#include <memory>

#include "ising.hpp"
#include "lattice.hpp"
