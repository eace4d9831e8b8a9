// ##################################################################
//
// main.cpp -- hamstr_gb300 executable (main.cpp:12-55 of the reference)
//
// Usage: hamstr_gb300 [case_dir]   (default: the working directory, which
// holds input.hamstr and input/domain000/ like the reference expects)
// ##################################################################
#include <cstdio>

#include "hamstr_host.h"

int main(int argc, char** argv)
{
   const std::string root = (argc > 1) ? argv[1] : "";
   try {
      HAMSTR ham(1, 0, root);
      ham.welcome();
      ham.readInputs(0);
      ham.preprocessor();
      ham.marchInTime();
      ham.thanks();
   } catch (const hamstr::Error& e) {
      std::fprintf(stderr, "hamstr_gb300: %s\n", e.what());
      return 1;
   }
   return 0;
}
