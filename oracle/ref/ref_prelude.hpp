/*
 * Forced-include prelude for building the reference's own sources as the
 * oracle (g++ -include oracle/ref/ref_prelude.hpp ...).  It stands in for the
 * reference's Definitions.hpp (same include guard, so that header is skipped)
 * with three differences that leave the reference's arithmetic untouched:
 *
 *  1. kN and kL become runtime constants, defined by the driver from the
 *     environment, so one binary serves every system size and box.
 *  2. std::normal_distribution is redirected to a distribution that returns
 *     the next value of an injected stream, in the reference's own draw order
 *     (the noise-injection hook: identical increments on both sides).
 *
 * No reference source is copied or edited.
 */
#ifndef SPC2ODEINTEGRATION_DEFINITIONS_HPP
#define SPC2ODEINTEGRATION_DEFINITIONS_HPP

#include <numeric>
#include <random>
#include <vector>

typedef double Real;
typedef float RealOutput;

extern const int kN;
const int kS = 3;
extern const Real kL;

extern std::mt19937 mersenne_twister_generator;

namespace spc_ref {
double next_injected_normal();
}

namespace std {
template <class RealType = double>
class spc_injected_normal_distribution {
 public:
  explicit spc_injected_normal_distribution(RealType = RealType(0), RealType = RealType(1)) {}
  template <class Generator>
  RealType operator()(Generator &) {
    return static_cast<RealType>(::spc_ref::next_injected_normal());
  }
};
}  // namespace std

#define normal_distribution spc_injected_normal_distribution

/*
 * 3. The observer's output folder.  BinaryObserver builds its file names from
 *    an absolute folder literal, `std::string file_folder("...")`
 *    (Observers/BinaryObserver.cpp:37-45).  This function-like macro rewrites
 *    that declaration only (a use of the name not followed by a parenthesis
 *    is left alone, and the macro does not expand inside its own expansion),
 *    so the files go to the folder the driver names (SPC_REF_OUT_DIR).
 */
namespace spc_ref {
const char *output_folder(const char *reference_folder);
}
#define file_folder(path) file_folder(::spc_ref::output_folder(path))

#endif
