// Empty stand-in for <GLFW/glfw3.h>: the reference's bvh.cpp includes it but
// calls nothing from it (its timers are commented out).  Test infrastructure
// for the oracle's reference build only.
#pragma once
