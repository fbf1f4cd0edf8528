// extern "C" access to the reference PL receiver's slot de-rotation
// (test infrastructure only; compiled into oracle/_ref by oracle/build.py).
// rotate_slot (plrx/pl_receiver.cc:1217-1282) lives in an anonymous
// namespace of that file, so this translation unit compiles the file itself,
// from where it lies in the reference tree, and forwards to the function.
#include "plrx/pl_receiver.cc"

extern "C" {

// one 90-symbol slot: o[i] = r[i] * d[i] * rot * step^i, the reference's
// four-chain evaluation (r, d, o: (re, im) float pairs)
void ref_rotate_slot(const float* r, const float* d, float rot_re, float rot_im, float step_re, float step_im,
                     float* o)
{
    using namespace cusat_dsp;
    rotate_slot(reinterpret_cast<const complexf*>(r), reinterpret_cast<const complexf*>(d),
                complexf(rot_re, rot_im), complexf(step_re, step_im), reinterpret_cast<complexf*>(o));
}

}  // extern "C"
