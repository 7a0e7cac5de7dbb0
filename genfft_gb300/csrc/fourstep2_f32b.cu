// fourstep2_f32b.cu -- the second half of the pair-packed four-step
// registrations (fourstep2_f32.cu), in its own translation unit so the two
// compile in parallel.
#define FS2_SET 1
#include "fourstep2_f32.cu"
