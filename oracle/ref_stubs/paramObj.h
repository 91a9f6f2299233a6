/* Stand-in for the SEP paramObj header (see genericIO.h in this folder). */
#pragma once
#include "genericIO.h"
