// Minimal stand-in for cereal 1.3.2's macros, so the reference compiles without cereal.
// Serialization is not on the measured or checked path; nothing here archives data.
#pragma once
#define CEREAL_SERIALIZE_FUNCTION_NAME serialize
#define CEREAL_LOAD_FUNCTION_NAME load
#define CEREAL_SAVE_FUNCTION_NAME save
#define CEREAL_NVP(x) (x)
