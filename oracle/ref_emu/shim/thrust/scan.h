#pragma once
#include "../thrust_emu.h"
