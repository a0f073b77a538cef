#pragma once
#include "colo_emu.h"
