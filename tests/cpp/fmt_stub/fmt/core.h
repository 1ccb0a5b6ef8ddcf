// Minimal stand-in for the fmt library (test infrastructure).
#pragma once
#include "format.h"
