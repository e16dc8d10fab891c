// ORACLE -- test infrastructure only: the serial cereal stand-in (cereal.hpp).
#pragma once
#include "cereal.hpp"
