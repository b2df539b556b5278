#include "ocaml_shim.h"
