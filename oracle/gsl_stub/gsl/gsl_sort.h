/* Header-only stand-in for GSL's sort header.  The reference's forward-model
 * header includes it but its dense path calls nothing from it.  Used only to
 * compile the reference sources as a test oracle in this repository. */
#ifndef GRADA_GSL_SORT_STUB_H
#define GRADA_GSL_SORT_STUB_H
#endif
