/* Reverse Cuthill-McKee on a sparse matrix, producing exactly the
 * permutation of the reference's dense bfm_perm_rcm (libbfm/src/perm.c:117-331).
 *
 * The ordering rules that make the result bit-exact:
 *   - a node's degree counts the nonzero entries of its row, diagonal included
 *     (perm.c:140-145); entries that are exactly 0.0 do not count;
 *   - each new BFS root is the unvisited index of minimum degree, taking the
 *     LAST such index on ties (perm.c:222-233, the `<=` comparison);
 *   - a popped node's unvisited neighbours are taken in ascending index order,
 *     marked visited at once, and pushed sorted by degree with a stable sort
 *     (perm.c:239-282: glibc's qsort is a stable merge sort);
 *   - the p-th popped node gets position n-1-p (perm.c:284).
 *
 * Cost: O(nnz + n log n) instead of the reference's O(n^2) scans.  Roots are
 * found by walking the nodes once in (degree ascending, index descending)
 * order, skipping visited ones.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <bfm/gpu.h>

typedef struct {
	int64_t i;
	int64_t deg;
} rcm_item_t;

static int64_t* g_deg_for_sort;

static int by_deg_then_index_desc(void const* a, void const* b) {
	int64_t const i = *(int64_t const*) a, j = *(int64_t const*) b;
	int64_t const di = g_deg_for_sort[i], dj = g_deg_for_sort[j];
	if (di != dj) return di < dj ? -1 : 1;
	return i > j ? -1 : (i < j ? 1 : 0);
}

/* stable insertion sort by degree (neighbour lists are short) */
static void stable_by_degree(rcm_item_t* v, int64_t n) {
	for (int64_t a = 1; a < n; a++) {
		rcm_item_t const t = v[a];
		int64_t b = a - 1;
		while (b >= 0 && v[b].deg > t.deg) {
			v[b + 1] = v[b];
			b--;
		}
		v[b + 1] = t;
	}
}

int bfm_gpu_rcm_csr(int64_t n, const int64_t* row_ptr, const int64_t* cols, const double* vals, int64_t* perm, int64_t* inv_perm) {
	if (n <= 0) return 0;
	int64_t* deg = calloc((size_t) n, sizeof *deg);
	int64_t* order = malloc((size_t) n * sizeof *order);
	unsigned char* visited = calloc((size_t) n, 1);
	int64_t* queue = malloc((size_t) n * sizeof *queue);
	int64_t max_row = 1;
	for (int64_t i = 0; i < n; i++)
		if (row_ptr[i + 1] - row_ptr[i] > max_row) max_row = row_ptr[i + 1] - row_ptr[i];
	rcm_item_t* nb = malloc((size_t) max_row * sizeof *nb);
	if (!deg || !order || !visited || !queue || !nb) {
		free(deg); free(order); free(visited); free(queue); free(nb);
		return -1;
	}
	for (int64_t i = 0; i < n; i++) {
		for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; k++) deg[i] += vals[k] != 0.0;
		order[i] = i;
	}
	/* qsort is only used on (degree, index) keys, which are all distinct */
	g_deg_for_sort = deg;
	qsort(order, (size_t) n, sizeof *order, by_deg_then_index_desc);
	g_deg_for_sort = NULL;

	int64_t head = 0, tail = 0, placed = 0, cursor = 0;
	while (placed < n) {
		while (visited[order[cursor]]) cursor++;
		int64_t const root = order[cursor];
		visited[root] = 1;
		queue[tail++] = root;
		while (head < tail) {
			int64_t const cur = queue[head++];
			int64_t cnt = 0;
			for (int64_t k = row_ptr[cur]; k < row_ptr[cur + 1]; k++) {
				int64_t const c = cols[k];
				if (visited[c] || vals[k] == 0.0) continue;
				visited[c] = 1;
				nb[cnt].i = c;
				nb[cnt].deg = deg[c];
				cnt++;
			}
			stable_by_degree(nb, cnt);
			for (int64_t k = 0; k < cnt; k++) queue[tail++] = nb[k].i;
			inv_perm[n - 1 - placed] = cur;
			placed++;
		}
	}
	for (int64_t i = 0; i < n; i++) perm[inv_perm[i]] = i;
	free(deg); free(order); free(visited); free(queue); free(nb);
	return 0;
}
