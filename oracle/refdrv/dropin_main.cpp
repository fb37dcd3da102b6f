// Driver of the linked drop-in boundary (test infrastructure, built only in
// the oracle's _ref/ tree): ref_inversion.cpp's main, renamed, with the
// reference's Fwd / GaussNewtonInversion / InversionBase / AdaptiveInversion
// members replaced by the drop-ins of graada3d_gb300/dropin/ at link time.
// A library error thrown by a drop-in (no GPU, a failing call) ends the run
// with exit status 7 and the message on stderr.
#include <cstdio>
#include <exception>

int ref_inversion_main(int argc, char **argv);

int main(int argc, char **argv) {
  try {
    return ref_inversion_main(argc, argv);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "drop-in: %s\n", e.what());
    return 7;
  }
}
