// AMReX header name the reference includes; everything it needs is in AMReX.H here.  Test infrastructure only.
#include "AMReX.H"
