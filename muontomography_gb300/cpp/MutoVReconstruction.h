// The reference's include/MutoVReconstruction.h: its class is declared, with the others of
// the reconstruction interface, in MutoReconstruction.h.  This header keeps
// the reference's include lines (its driver MuToTest.cpp includes one header
// per class) compiling unchanged against this library.
#pragma once

#include "MutoReconstruction.h"
