// Stand-in for libcua's header of this name (test infrastructure only).
#pragma once
#include "cua_emu.h"
