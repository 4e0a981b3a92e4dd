// compile-only stand-in (see chroma_stand_in.h)
#pragma once
#include "../../../chroma_stand_in.h"
