// Host-side helpers shared by the one-system API (api.cu) and the batched
// API (batch.cu).
#pragma once

#include <string>

#include "../../include/pimdb_gb300.h"
#include "common.cuh"

// Empty when the configuration is usable, else the reason (the reference's
// wording where it has one: src/params.cpp:8-260).
std::string validate_config(const pimdb_config& c);
// Scalar parameters of one system from its configuration (device pointers
// untouched).
void sys_params_from_config(const pimdb_config& c, pimdb::Sys& s);
