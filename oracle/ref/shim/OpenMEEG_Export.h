#pragma once
#define OPENMEEG_EXPORT __attribute__((visibility("default")))
