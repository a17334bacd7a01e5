/* ORACLE TEST INFRASTRUCTURE -- not part of the product.
 *
 * Minimal stand-in for the arena allocator of the external "cop" library
 * (github.com/nickappleton/cop, not vendored by fftset, no pinned version).
 * It exists only so the unmodified fftset sources can be compiled here as a
 * checker. Semantics are taken from fftset's call sites:
 *   fftset.h:24,165-166        struct types embedded in struct fftset
 *   src/fftset.c:84            cop_alloc_grp_temps_init(grp, iface, initial, max, align) -> 0 on success
 *   src/fftset.c:94            cop_alloc_grp_temps_free(grp) frees every allocation
 *   src/fftset.c:111, src/fftset_vec.c:1071,1090
 *                              cop_salloc(iface, size, align) -> aligned block or NULL
 * Every block is kept on a singly linked list owned by the group. */
#ifndef ORACLE_COP_ALLOC_H
#define ORACLE_COP_ALLOC_H

#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>

struct oracle_cop_block {
	struct oracle_cop_block *next;
};

struct cop_alloc_grp_temps {
	struct oracle_cop_block *blocks;
	size_t                   align;
};

struct cop_salloc_iface {
	struct cop_alloc_grp_temps *grp;
};

static inline int
cop_alloc_grp_temps_init(struct cop_alloc_grp_temps *grp, struct cop_salloc_iface *iface, size_t initial, size_t max, size_t align)
{
	(void)initial;
	(void)max;
	grp->blocks = NULL;
	grp->align  = align ? align : 16;
	iface->grp  = grp;
	return 0;
}

static inline void *
cop_salloc(struct cop_salloc_iface *iface, size_t size, size_t align)
{
	size_t a = align ? align : iface->grp->align;
	char *raw;
	uintptr_t p;
	if (a < 64)
		a = 64;
	raw = (char *)malloc(sizeof(struct oracle_cop_block) + size + a);
	if (raw == NULL)
		return NULL;
	((struct oracle_cop_block *)raw)->next = iface->grp->blocks;
	iface->grp->blocks = (struct oracle_cop_block *)raw;
	p = (uintptr_t)(raw + sizeof(struct oracle_cop_block));
	p = (p + a - 1) & ~(uintptr_t)(a - 1);
	return (void *)p;
}

static inline void
cop_alloc_grp_temps_free(struct cop_alloc_grp_temps *grp)
{
	while (grp->blocks != NULL) {
		struct oracle_cop_block *n = grp->blocks->next;
		free(grp->blocks);
		grp->blocks = n;
	}
}

#endif
