// Serialization is only needed for inter-process transfer, which a single-GPU process does not do;
// this header exists so that code including it compiles unchanged.
#pragma once
