#pragma once
#include "af_emu.h"
