// Stand-in declarations for the tinyexpr library (driver motion expressions,
// never evaluated by the harness).
#pragma once
#include <cassert>
#include <string>
struct te_expr;
struct te_variable {
  const char* name;
  const void* address;
};
te_expr* te_compile(const char* expression, const te_variable* variables, int var_count, int* error);
double te_eval(const te_expr* n);
void te_free(te_expr* n);
