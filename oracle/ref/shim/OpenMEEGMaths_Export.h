#pragma once
#define OPENMEEGMATHS_EXPORT __attribute__((visibility("default")))
