/* ORACLE TEST INFRASTRUCTURE -- not part of the product.
 * Helpers compiled together with the unmodified reference sources so that
 * Python (ctypes) can drive them: struct fftset is caller-allocated in the
 * reference API (fftset.h:159-167), so it is heap-allocated here. */
#include <stdlib.h>
#include "fftset/fftset.h"

struct fftset *oref_new(void)
{
	struct fftset *f = (struct fftset *)malloc(sizeof(*f));
	if (f != NULL && fftset_init(f)) {
		free(f);
		f = NULL;
	}
	return f;
}

void oref_free(struct fftset *f)
{
	if (f != NULL) {
		fftset_destroy(f);
		free(f);
	}
}

const struct fftset_modulation *oref_modulation(int freq_offset_real)
{
	return freq_offset_real ? FFTSET_MODULATION_FREQ_OFFSET_REAL : FFTSET_MODULATION_COMPLEX;
}
