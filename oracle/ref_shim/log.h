// Stand-in for the proprietary engine's log.h included by src/utils/timer.h.
#pragma once
#include <string>
