/* Persistent autotune results (no reference counterpart: the reference
 * plans inside fftset_create_fft, src/fftset_vec.c:993-1152, and keeps
 * nothing across processes).
 *
 * fftset_tuning_save writes, for every plan of an fftset, the compiled
 * kernel variant selected per operation (fftset_fft_autotune or
 * fftset_fft_set_variant) and the task-kernel schedule fftset_ragged_autotune
 * picked; fftset_tuning_load creates the same plans in another fftset (in
 * another process) and applies those choices, so a service tunes once per
 * device model and reuses the result. Text, one record per line:
 *
 *   fftset-tuning 1
 *   device <multiprocessors> <device name>
 *   fft <modulation: 0 COMPLEX, 1 FREQ_OFFSET_REAL> <complex_bins> <variant per op, FGK_OP_* order>
 *   ragged <modulation> <complex_bins> <stages> <radix>... <threads per item> <ls1> <ls2>
 *
 * (variant -1 is the generic kernel; ragged stages 0 is the plan's own
 * chain). A file written on another device model is refused with
 * FFTSET_E_UNSUPPORTED before anything is applied; a malformed or
 * inconsistent record stops the load with FFTSET_E_INVALID (records before it
 * stay applied). */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "fftset.h"
#include "fftset_internal.h"

#define FST_MAGIC "fftset-tuning 1"

static int fst_device(struct fs_impl *fs, char *name, size_t cap, int *sms)
{
	struct cudaDeviceProp prop;
	size_t i;
	if (cudaGetDeviceProperties(&prop, fs->device) != cudaSuccess) {
		cudaGetLastError();
		return FFTSET_E_CUDA;
	}
	snprintf(name, cap, "%s", prop.name);
	for (i = 0; name[i]; i++)
		if (name[i] == '\n' || name[i] == '\r')
			name[i] = ' ';
	*sms = prop.multiProcessorCount;
	return FFTSET_OK;
}

int fftset_tuning_save(struct fftset *fc, const char *path)
{
	struct fs_impl *fs = fs_impl_of(fc);
	const struct fftset_fft *f;
	char name[256];
	int sms, rc, op;
	FILE *fp;
	if (!fs || !path)
		return FFTSET_E_INVALID;
	if ((rc = fst_device(fs, name, sizeof(name), &sms)) != FFTSET_OK)
		return fs_latch(fs, rc, 0);
	if (!(fp = fopen(path, "w")))
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	fprintf(fp, "%s\ndevice %d %s\n", FST_MAGIC, sms, name);
	for (f = fs->first; f; f = f->next) {
		const int mod = f->modulator->freq_offset_real ? 1 : 0;
		fprintf(fp, "fft %d %u", mod, f->lfft);
		for (op = 0; op < FGK_OP_COUNT; op++)
			fprintf(fp, " %d", f->sel[op]);
		fputc('\n', fp);
		if (f->rg_tuned) {
			/* the chain only when it is not the plan's own */
			uint32_t s, n = f->rg_plan.fwd.nstages, own = n == f->rp.fwd.nstages;
			for (s = 0; own && s < n; s++)
				own = f->rg_plan.fwd.st[s].radix == f->rp.fwd.st[s].radix;
			if (!f->rg_dmem || own)
				n = 0;
			fprintf(fp, "ragged %d %u %u", mod, f->lfft, n);
			for (s = 0; s < n; s++)
				fprintf(fp, " %u", f->rg_plan.fwd.st[s].radix);
			fprintf(fp, " %u %u %u\n", f->rg_tg, f->rg_ls1, f->rg_ls2);
		}
	}
	rc = ferror(fp) ? FFTSET_E_INVALID : FFTSET_OK;
	if (fclose(fp) != 0)
		rc = FFTSET_E_INVALID;
	return rc ? fs_latch(fs, rc, 0) : FFTSET_OK;
}

/* next whitespace-separated unsigned / signed integer of *p */
static int fst_uint(char **p, unsigned *v)
{
	char *e;
	unsigned long x = strtoul(*p, &e, 10);
	if (e == *p || x > 0xffffffffUL)
		return 0;
	*v = (unsigned)x;
	*p = e;
	return 1;
}

static int fst_int(char **p, int *v)
{
	char *e;
	long x = strtol(*p, &e, 10);
	if (e == *p || x < -1 || x > 1000)
		return 0;
	*v = (int)x;
	*p = e;
	return 1;
}

static const struct fftset_modulation *fst_mod(unsigned m)
{
	return m == 0 ? FFTSET_MODULATION_COMPLEX : m == 1 ? FFTSET_MODULATION_FREQ_OFFSET_REAL : NULL;
}

/* one record after its keyword; returns FFTSET_OK or an error code */
static int fst_record(struct fs_impl *fs, const char *kw, char *p)
{
	unsigned m, L;
	struct fftset_fft *f;
	if (!fst_uint(&p, &m) || !fst_uint(&p, &L) || !fst_mod(m))
		return FFTSET_E_INVALID;
	if (!(f = fs_create_plan(fs, fst_mod(m), L)))
		return FFTSET_E_INVALID;
	if (strcmp(kw, "fft") == 0) {
		int sel[FGK_OP_COUNT], op;
		for (op = 0; op < FGK_OP_COUNT; op++) {
			if (!fst_int(&p, &sel[op]) || sel[op] >= f->nvar ||
			    (sel[op] >= 0 && !(f->vops[sel[op]] & (1u << op))))
				return FFTSET_E_INVALID;
		}
		for (op = 0; op < FGK_OP_COUNT; op++)
			f->sel[op] = sel[op];
		return FFTSET_OK;
	} else {
		uint32_t rad[FGK_MAX_STAGES];
		unsigned n, s, tg, ls1, ls2, prod = 1;
		if (!fst_uint(&p, &n) || n > FGK_MAX_STAGES)
			return FFTSET_E_INVALID;
		for (s = 0; s < n; s++) {
			unsigned r;
			if (!fst_uint(&p, &r) || r < 2 || r > 16)
				return FFTSET_E_INVALID;
			rad[s] = r;
			prod *= r;
		}
		if ((n && prod != L) || !fst_uint(&p, &tg) || !fst_uint(&p, &ls1) || !fst_uint(&p, &ls2))
			return FFTSET_E_INVALID;
		return fsr_apply_schedule(fs, f, rad, n, tg, ls1, ls2);
	}
}

int fftset_tuning_load(struct fftset *fc, const char *path)
{
	struct fs_impl *fs = fs_impl_of(fc);
	char line[1024], name[256];
	int sms, rc, lineno = 0;
	FILE *fp;
	if (!fs || !path)
		return FFTSET_E_INVALID;
	if ((rc = fst_device(fs, name, sizeof(name), &sms)) != FFTSET_OK)
		return fs_latch(fs, rc, 0);
	if (!(fp = fopen(path, "r")))
		return fs_latch(fs, FFTSET_E_INVALID, 0);
	rc = FFTSET_OK;
	while (rc == FFTSET_OK && fgets(line, sizeof(line), fp)) {
		char *p = line, *kw;
		size_t n = strlen(line);
		if (n && line[n - 1] == '\n')
			line[--n] = 0;
		if (++lineno == 1) {
			rc = strcmp(line, FST_MAGIC) == 0 ? FFTSET_OK : FFTSET_E_INVALID;
			continue;
		}
		while (*p == ' ')
			p++;
		if ((!*p || *p == '#') && lineno > 2)
			continue;
		kw = p;
		while (*p && *p != ' ')
			p++;
		if (*p)
			*p++ = 0;
		if (lineno == 2) { /* the device line comes first: nothing is applied for another model */
			unsigned fsms;
			if (strcmp(kw, "device") != 0 || !fst_uint(&p, &fsms))
				rc = FFTSET_E_INVALID;
			else if ((int)fsms != sms || strcmp(p + (*p == ' '), name) != 0)
				rc = FFTSET_E_UNSUPPORTED; /* tuned on another device model */
		} else if (strcmp(kw, "fft") == 0 || strcmp(kw, "ragged") == 0) {
			rc = fst_record(fs, kw, p);
		} else {
			rc = FFTSET_E_INVALID;
		}
	}
	if (rc == FFTSET_OK && lineno < 2)
		rc = FFTSET_E_INVALID; /* no device line */
	fclose(fp);
	return rc ? fs_latch(fs, rc, 0) : FFTSET_OK;
}
