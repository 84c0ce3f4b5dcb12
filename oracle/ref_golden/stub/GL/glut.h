/* See glew.h: compile-only stand-in, no windowing functions are provided. */
#pragma once
#include "glew.h"
