/*
 * bfs_oracle.c -- CPU oracle for the GraphPhi hybrid BFS path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C with OpenMP, the
 * algorithm of the reference's hybrid top-down/bottom-up BFS
 * (apps/bfs_simd/bfs.cpp, apps/bfs_serial/bfs.cpp) and of the preprocessing
 * tools that write its input files (tools/csr_tiling, tools/coo_tiling,
 * tools/column_major_tile, tools/vertex_id_remap).  It is the checker the GPU
 * product is compared against and the CPU baseline that bench.py times; the
 * product never links, loads or calls it.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference legs may use it.
 *
 * Every function cites the reference lines it follows.  The restatement keeps
 * the reference's data layout (unsigned 32-bit ids, int flag arrays, int cost,
 * unsigned parents with (unsigned)-1 for "unvisited") and its control flow,
 * with the AVX-512 intrinsics replaced by the scalar loops that bfs_serial
 * uses for the same steps.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#define ORC_OK 0
#define ORC_EIO 1
#define ORC_EFORMAT 2
#define ORC_ENOMEM 3
#define ORC_EARG 4

#define ORC_NUM_FILES 64 /* 64-way split, e.g. tools/csr_tiling/page_rank.cpp:571 */
#define UNVISITED ((unsigned) -1)

/* ------------------------------------------------------------------------ */
/* Small helpers                                                            */
/* ------------------------------------------------------------------------ */

static unsigned side_length_of(unsigned n, unsigned w)
{
	/* apps/bfs_simd/bfs.cpp:995-999 */
	return (n % w) ? n / w + 1 : n / w;
}

/* Edge index range held by split file `tid` (apps/bfs_simd/bfs.cpp:1025-1044). */
static void split_range(unsigned m, unsigned tid, unsigned *lo, unsigned *hi)
{
	unsigned bound = m / ORC_NUM_FILES;
	*lo = tid * bound;
	*hi = (tid != ORC_NUM_FILES - 1) ? *lo + bound : m;
}

/* ------------------------------------------------------------------------ */
/* In-memory restatement of the preprocessing tools                          */
/* ------------------------------------------------------------------------ */

/*
 * CSR order: edges bucketed by source in input order
 * (tools/csr_tiling/page_rank.cpp:531-567, input_untiled; no dedup, no
 * self-loop removal).  0-based ids in and out.  `degrees` gets the out-degree
 * of every vertex (the _untiled-nneibor file, :594-598).
 */
int orc_csr_order(unsigned n, unsigned m, const unsigned *src, const unsigned *dst,
		unsigned *out_src, unsigned *out_dst, unsigned *degrees)
{
	unsigned *start = (unsigned *) malloc(sizeof(unsigned) * ((size_t) n + 1));
	if (!start) return ORC_ENOMEM;
	memset(degrees, 0, sizeof(unsigned) * n);
	for (unsigned i = 0; i < m; ++i) {
		if (src[i] >= n || dst[i] >= n) { free(start); return ORC_EFORMAT; }
		degrees[src[i]]++;
	}
	unsigned acc = 0;
	for (unsigned v = 0; v < n; ++v) { start[v] = acc; acc += degrees[v]; }
	for (unsigned i = 0; i < m; ++i) {
		unsigned pos = start[src[i]]++;
		out_src[pos] = src[i];
		out_dst[pos] = dst[i];
	}
	free(start);
	return ORC_OK;
}

/*
 * Row-major 2-D COO tiles: tile_id = (u/W)*SIDE + v/W, edges keep their CSR
 * order inside a tile (tools/coo_tiling/page_rank.cpp:404-447); tile_offsets
 * has SIDE*SIDE entries, the first edge index of each tile (:488-495).
 */
int orc_coo_tile_order(unsigned n, unsigned m, const unsigned *src, const unsigned *dst,
		unsigned w, unsigned *out_src, unsigned *out_dst, unsigned *tile_offsets)
{
	unsigned side = side_length_of(n, w);
	size_t num_tiles = (size_t) side * side;
	unsigned *fill = (unsigned *) calloc(num_tiles + 1, sizeof(unsigned));
	if (!fill) return ORC_ENOMEM;
	for (unsigned i = 0; i < m; ++i) {
		size_t t = (size_t) (src[i] / w) * side + dst[i] / w;
		fill[t + 1]++;
	}
	for (size_t t = 0; t < num_tiles; ++t) fill[t + 1] += fill[t];
	for (size_t t = 0; t < num_tiles; ++t) tile_offsets[t] = fill[t];
	for (unsigned i = 0; i < m; ++i) {
		size_t t = (size_t) (src[i] / w) * side + dst[i] / w;
		unsigned pos = fill[t]++;
		out_src[pos] = src[i];
		out_dst[pos] = dst[i];
	}
	free(fill);
	return ORC_OK;
}

/*
 * Column-major stripes: for side_i in steps of S, for col, for row in the
 * stripe; then a tail stripe of the remaining SIDE-side_i rows
 * (tools/column_major_tile/kcore.cpp:360-415).  The new offsets are indexed by
 * the position of the tile in that order.
 */
int orc_col_major_order(unsigned n, unsigned m, const unsigned *src, const unsigned *dst,
		const unsigned *tile_offsets, unsigned w, unsigned s,
		unsigned *out_src, unsigned *out_dst, unsigned *out_offsets)
{
	unsigned side = side_length_of(n, w);
	size_t num_tiles = (size_t) side * side;
	unsigned edge_index = 0;
	size_t new_tile_id = 0;
	unsigned side_i;
	for (side_i = 0; side_i + s <= side; side_i += s) {
		for (unsigned col = 0; col < side; ++col) {
			for (unsigned row = side_i; row < side_i + s; ++row) {
				size_t tile_id = (size_t) row * side + col;
				unsigned bound = (tile_id != num_tiles - 1) ? tile_offsets[tile_id + 1] : m;
				out_offsets[new_tile_id++] = edge_index;
				for (unsigned e = tile_offsets[tile_id]; e < bound; ++e) {
					out_src[edge_index] = src[e];
					out_dst[edge_index] = dst[e];
					++edge_index;
				}
			}
		}
	}
	if (side_i != side) {
		for (unsigned col = 0; col < side; ++col) {
			for (unsigned row = side_i; row < side; ++row) {
				size_t tile_id = (size_t) row * side + col;
				unsigned bound = (tile_id != num_tiles - 1) ? tile_offsets[tile_id + 1] : m;
				out_offsets[new_tile_id++] = edge_index;
				for (unsigned e = tile_offsets[tile_id]; e < bound; ++e) {
					out_src[edge_index] = src[e];
					out_dst[edge_index] = dst[e];
					++edge_index;
				}
			}
		}
	}
	return (edge_index == m && new_tile_id == num_tiles) ? ORC_OK : ORC_EFORMAT;
}

/*
 * BFS-discovery relabelling from vertex 0 (tools/vertex_id_remap/bfs.cpp):
 * Rodinia-style level-synchronous BFS over the CSR (:493-552); after each
 * level the newly reached vertices get the next labels in ascending old id
 * (add_mask2map, :465-479); unreached vertices are labelled last in ascending
 * old id (add_remainder2map, :481-491).  vertex_map[old] = new.
 */
int orc_vertex_remap_map(unsigned n, const unsigned *row_start, const unsigned *degrees,
		const unsigned *edges, unsigned *vertex_map)
{
	int *mask = (int *) calloc(n, sizeof(int));
	int *updating = (int *) calloc(n, sizeof(int));
	int *visited = (int *) calloc(n, sizeof(int));
	if (!mask || !updating || !visited) { free(mask); free(updating); free(visited); return ORC_ENOMEM; }
	for (unsigned i = 0; i < n; ++i) vertex_map[i] = UNVISITED;
	unsigned top = 0;
	const unsigned source = 0;
	if (n == 0) { free(mask); free(updating); free(visited); return ORC_OK; }
	vertex_map[source] = top++;
	mask[source] = 1;
	visited[source] = 1;
	int stop;
	do {
		stop = 1;
		for (unsigned u = 0; u < n; ++u) {
			if (mask[u] != 1) continue;
			mask[u] = 0;
			for (unsigned e = row_start[u]; e < row_start[u] + degrees[u]; ++e) {
				unsigned v = edges[e];
				if (!visited[v]) updating[v] = 1;
			}
		}
		for (unsigned v = 0; v < n; ++v)
			if (updating[v]) vertex_map[v] = top++;
		for (unsigned v = 0; v < n; ++v) {
			if (updating[v] == 1) {
				mask[v] = 1;
				visited[v] = 1;
				stop = 0;
				updating[v] = 0;
			}
		}
	} while (!stop);
	for (unsigned v = 0; v < n; ++v)
		if (vertex_map[v] == UNVISITED) vertex_map[v] = top++;
	free(mask); free(updating); free(visited);
	return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Text files                                                               */
/* ------------------------------------------------------------------------ */

/*
 * Writes the 64-way split family <prefix>-0..63: "N M\n" at the top of file 0,
 * then file t holds edges [t*floor(M/64), ...) as 1-indexed "u v\n" lines, or
 * "u v w\n" when weights != NULL (tools/csr_tiling/page_rank.cpp:570-592,
 * :474-496; tools/coo_tiling/page_rank.cpp:452-485;
 * tools/column_major_tile/kcore.cpp:419-441).
 */
int orc_write_split(const char *prefix, unsigned n, unsigned m, const unsigned *a,
		const unsigned *b, const unsigned *weights)
{
	char name[4096];
	for (unsigned tid = 0; tid < ORC_NUM_FILES; ++tid) {
		unsigned lo, hi;
		split_range(m, tid, &lo, &hi);
		snprintf(name, sizeof(name), "%s-%u", prefix, tid);
		FILE *f = fopen(name, "w");
		if (!f) return ORC_EIO;
		if (tid == 0) fprintf(f, "%u %u\n", n, m);
		for (unsigned i = lo; i < hi; ++i) {
			if (weights) fprintf(f, "%u %u %u\n", a[i] + 1, b[i] + 1, weights[i]);
			else fprintf(f, "%u %u\n", a[i] + 1, b[i] + 1);
		}
		fclose(f);
	}
	return ORC_OK;
}

/* One "%u\n" per entry: -offsets and -nneibor files (coo_tiling :488-501). */
int orc_write_lines(const char *path, const unsigned *v, size_t count)
{
	FILE *f = fopen(path, "w");
	if (!f) return ORC_EIO;
	for (size_t i = 0; i < count; ++i) fprintf(f, "%u\n", v[i]);
	fclose(f);
	return ORC_OK;
}

/* Edge list "N M\n" + 1-indexed "u v\n" lines (README.md:19-24 input format,
 * and the single _reorder file of tools/vertex_id_remap/bfs.cpp:50-63). */
int orc_write_edge_list(const char *path, unsigned n, unsigned m, const unsigned *src,
		const unsigned *dst, const unsigned *weights)
{
	FILE *f = fopen(path, "w");
	if (!f) return ORC_EIO;
	fprintf(f, "%u %u\n", n, m);
	for (unsigned i = 0; i < m; ++i) {
		if (weights) fprintf(f, "%u %u %u\n", src[i] + 1, dst[i] + 1, weights[i]);
		else fprintf(f, "%u %u\n", src[i] + 1, dst[i] + 1);
	}
	fclose(f);
	return ORC_OK;
}

/* Reads "N M" from the head of a file (apps/bfs_simd/bfs.cpp:987-994). */
int orc_read_header(const char *path, unsigned *n, unsigned *m)
{
	FILE *f = fopen(path, "r");
	if (!f) return ORC_EIO;
	int ok = fscanf(f, "%u %u", n, m) == 2;
	fclose(f);
	return ok ? ORC_OK : ORC_EFORMAT;
}

/* Reads an edge-list file written by orc_write_edge_list into 0-based arrays. */
int orc_read_edge_list(const char *path, unsigned m, unsigned *src, unsigned *dst, int weighted)
{
	FILE *f = fopen(path, "r");
	if (!f) return ORC_EIO;
	unsigned n0, m0, w;
	if (fscanf(f, "%u %u", &n0, &m0) != 2 || m0 != m) { fclose(f); return ORC_EFORMAT; }
	for (unsigned i = 0; i < m; ++i) {
		unsigned a, b;
		if (fscanf(f, "%u %u", &a, &b) != 2) { fclose(f); return ORC_EFORMAT; }
		if (weighted && fscanf(f, "%u", &w) != 1) { fclose(f); return ORC_EFORMAT; }
		src[i] = a - 1;
		dst[i] = b - 1;
	}
	fclose(f);
	return ORC_OK;
}

/*
 * Reads the 64-way split family into 0-based arrays (apps/bfs_simd/bfs.cpp
 * :1021-1056 for heads/tails, :1076-1106 for the CSR destinations, where only
 * b is kept).  a may be NULL.  weighted files carry a third column that is
 * dropped.
 */
int orc_read_split(const char *prefix, unsigned m, unsigned *a, unsigned *b, int weighted)
{
	char name[4096];
	int status = ORC_OK;
#pragma omp parallel for schedule(static, 1)
	for (unsigned tid = 0; tid < ORC_NUM_FILES; ++tid) {
		unsigned lo, hi, n0, m0, w;
		split_range(m, tid, &lo, &hi);
		char fname[4096];
		snprintf(fname, sizeof(fname), "%s-%u", prefix, tid);
		FILE *f = fopen(fname, "r");
		if (!f) {
#pragma omp atomic write
			status = ORC_EIO;
			continue;
		}
		if (tid == 0 && fscanf(f, "%u %u", &n0, &m0) != 2) {
#pragma omp atomic write
			status = ORC_EFORMAT;
		}
		for (unsigned i = lo; i < hi; ++i) {
			unsigned x, y;
			if (fscanf(f, "%u %u", &x, &y) != 2 || (weighted && fscanf(f, "%u", &w) != 1)) {
#pragma omp atomic write
				status = ORC_EFORMAT;
				break;
			}
			if (a) a[i] = x - 1;
			b[i] = y - 1;
		}
		fclose(f);
	}
	(void) name;
	return status;
}

/* Reads `count` "%u" values (the -offsets / -nneibor files, bfs.cpp:1002-1012, :1065-1074). */
int orc_read_lines(const char *path, unsigned *v, size_t count)
{
	FILE *f = fopen(path, "r");
	if (!f) return ORC_EIO;
	for (size_t i = 0; i < count; ++i) {
		if (fscanf(f, "%u", v + i) != 1) { fclose(f); return ORC_EFORMAT; }
	}
	fclose(f);
	return ORC_OK;
}

/*
 * The ONEDEBUG level dump: 64 files <dir>/path<t>.txt, each with lines
 * "<v>) cost:<level>\n" for floor(N/64) vertices, the last file taking the rest
 * (apps/bfs_simd/bfs.cpp:927-954).
 */
int orc_write_path_dump(const char *dir, unsigned n, const int *cost)
{
	unsigned num_lines = n / 64;
	char name[4096];
	for (unsigned tid = 0; tid < 64; ++tid) {
		unsigned lo = tid * num_lines;
		unsigned hi = (tid != 63) ? lo + num_lines : n;
		snprintf(name, sizeof(name), "%s/path%u.txt", dir, tid);
		FILE *f = fopen(name, "w");
		if (!f) return ORC_EIO;
		for (unsigned v = lo; v < hi; ++v) fprintf(f, "%d) cost:%d\n", (int) v, cost[v]);
		fclose(f);
	}
	return ORC_OK;
}

/* Reads a dump written by orc_write_path_dump (or by the reference) back. */
int orc_read_path_dump(const char *dir, unsigned n, int *cost)
{
	unsigned num_lines = n / 64;
	char name[4096];
	for (unsigned tid = 0; tid < 64; ++tid) {
		unsigned lo = tid * num_lines;
		unsigned hi = (tid != 63) ? lo + num_lines : n;
		snprintf(name, sizeof(name), "%s/path%u.txt", dir, tid);
		FILE *f = fopen(name, "r");
		if (!f) return ORC_EIO;
		for (unsigned v = lo; v < hi; ++v) {
			int idx, c;
			if (fscanf(f, "%d) cost:%d", &idx, &c) != 2 || (unsigned) idx != v) { fclose(f); return ORC_EFORMAT; }
			cost[v] = c;
		}
		fclose(f);
	}
	return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Whole-tool restatements (the CLIs of the tools)                         */
/* ------------------------------------------------------------------------ */

/* tools/csr_tiling/page_rank.cpp main + input_untiled / input_weighted. */
int orc_tool_csr_tiling(const char *edge_list, int weighted)
{
	unsigned n, m;
	int st = orc_read_header(edge_list, &n, &m);
	if (st) return st;
	unsigned *src = malloc(sizeof(unsigned) * (size_t) m + 4), *dst = malloc(sizeof(unsigned) * (size_t) m + 4);
	unsigned *cs = malloc(sizeof(unsigned) * (size_t) m + 4), *cd = malloc(sizeof(unsigned) * (size_t) m + 4);
	unsigned *deg = malloc(sizeof(unsigned) * (size_t) n + 4);
	unsigned *wt = NULL, *cw = NULL;
	if (!src || !dst || !cs || !cd || !deg) { st = ORC_ENOMEM; goto out; }
	if (weighted) {
		/* Weighted edges keep their weight through the bucketing (:440-471). */
		wt = malloc(sizeof(unsigned) * (size_t) m + 4);
		cw = malloc(sizeof(unsigned) * (size_t) m + 4);
		FILE *f = fopen(edge_list, "r");
		if (!f || !wt || !cw) { st = ORC_EIO; if (f) fclose(f); goto out; }
		unsigned n0, m0;
		if (fscanf(f, "%u %u", &n0, &m0) != 2) { fclose(f); st = ORC_EFORMAT; goto out; }
		for (unsigned i = 0; i < m; ++i) {
			if (fscanf(f, "%u %u %u", src + i, dst + i, wt + i) != 3) { fclose(f); st = ORC_EFORMAT; goto out; }
			src[i]--; dst[i]--;
		}
		fclose(f);
	} else {
		st = orc_read_edge_list(edge_list, m, src, dst, 0);
		if (st) goto out;
	}
	st = orc_csr_order(n, m, src, dst, cs, cd, deg);
	if (st) goto out;
	if (weighted) {
		/* The weight follows its edge: redo the stable bucketing for weights. */
		unsigned *start = malloc(sizeof(unsigned) * ((size_t) n + 1));
		unsigned acc = 0;
		for (unsigned v = 0; v < n; ++v) { start[v] = acc; acc += deg[v]; }
		for (unsigned i = 0; i < m; ++i) cw[start[src[i]]++] = wt[i];
		free(start);
	}
	{
		char prefix[4096];
		snprintf(prefix, sizeof(prefix), "%s_untiled", edge_list);
		st = orc_write_split(prefix, n, m, cs, cd, cw);
		if (st) goto out;
		char nb[4200];
		snprintf(nb, sizeof(nb), "%s-nneibor", prefix);
		st = orc_write_lines(nb, deg, n);
	}
out:
	free(src); free(dst); free(cs); free(cd); free(deg); free(wt); free(cw);
	return st;
}

/* tools/coo_tiling/page_rank.cpp input_data (:324-515), one tile width per call
 * (the tool loops min..max doubling, :399). */
int orc_tool_coo_tiling(const char *base, unsigned w)
{
	char prefix[4096], name[4200];
	unsigned n, m;
	snprintf(prefix, sizeof(prefix), "%s_untiled", base);
	snprintf(name, sizeof(name), "%s-0", prefix);
	int st = orc_read_header(name, &n, &m);
	if (st) return st;
	unsigned side = side_length_of(n, w);
	size_t num_tiles = (size_t) side * side;
	unsigned *s = malloc(4 * (size_t) m + 4), *d = malloc(4 * (size_t) m + 4);
	unsigned *ts = malloc(4 * (size_t) m + 4), *td = malloc(4 * (size_t) m + 4);
	unsigned *off = malloc(4 * num_tiles + 4), *deg = calloc((size_t) n + 1, 4);
	if (!s || !d || !ts || !td || !off || !deg) { st = ORC_ENOMEM; goto out; }
	st = orc_read_split(prefix, m, s, d, 0);
	if (st) goto out;
	for (unsigned i = 0; i < m; ++i) deg[s[i]]++; /* nneibor, :431 */
	st = orc_coo_tile_order(n, m, s, d, w, ts, td, off);
	if (st) goto out;
	snprintf(prefix, sizeof(prefix), "%s_coo-tiled-%u", base, w);
	st = orc_write_split(prefix, n, m, ts, td, NULL);
	if (st) goto out;
	snprintf(name, sizeof(name), "%s-offsets", prefix);
	st = orc_write_lines(name, off, num_tiles);
	if (st) goto out;
	snprintf(name, sizeof(name), "%s-nneibor", prefix);
	st = orc_write_lines(name, deg, n);
out:
	free(s); free(d); free(ts); free(td); free(off); free(deg);
	return st;
}

/* tools/column_major_tile/kcore.cpp input (:143-244) + convert_to_col_major
 * (:360-467), one stripe length per call (the tool loops min..max doubling). */
int orc_tool_column_major(const char *base, unsigned w, unsigned stripe)
{
	char prefix[4096], name[4200];
	unsigned n, m;
	snprintf(prefix, sizeof(prefix), "%s_coo-tiled-%u", base, w);
	snprintf(name, sizeof(name), "%s-0", prefix);
	int st = orc_read_header(name, &n, &m);
	if (st) return st;
	unsigned side = side_length_of(n, w);
	size_t num_tiles = (size_t) side * side;
	unsigned *s = malloc(4 * (size_t) m + 4), *d = malloc(4 * (size_t) m + 4);
	unsigned *cs = malloc(4 * (size_t) m + 4), *cd = malloc(4 * (size_t) m + 4);
	unsigned *off = malloc(4 * num_tiles + 4), *noff = malloc(4 * num_tiles + 4);
	unsigned *deg = malloc(4 * (size_t) n + 4);
	if (!s || !d || !cs || !cd || !off || !noff || !deg) { st = ORC_ENOMEM; goto out; }
	snprintf(name, sizeof(name), "%s-offsets", prefix);
	if ((st = orc_read_lines(name, off, num_tiles))) goto out;
	snprintf(name, sizeof(name), "%s-nneibor", prefix);
	if ((st = orc_read_lines(name, deg, n))) goto out;
	if ((st = orc_read_split(prefix, m, s, d, 0))) goto out;
	if ((st = orc_col_major_order(n, m, s, d, off, w, stripe, cs, cd, noff))) goto out;
	snprintf(prefix, sizeof(prefix), "%s_col-%u-coo-tiled-%u", base, stripe, w);
	if ((st = orc_write_split(prefix, n, m, cs, cd, NULL))) goto out;
	snprintf(name, sizeof(name), "%s-offsets", prefix);
	if ((st = orc_write_lines(name, noff, num_tiles))) goto out;
	snprintf(name, sizeof(name), "%s-nneibor", prefix);
	st = orc_write_lines(name, deg, n);
out:
	free(s); free(d); free(cs); free(cd); free(off); free(noff); free(deg);
	return st;
}

/* tools/vertex_id_remap/bfs.cpp BFSGraph (:69-247): reads <base>_untiled-*,
 * writes <base>_reorder with the CSR-ordered edges relabelled (make_up_data, :42-64). */
int orc_tool_vertex_remap(const char *base)
{
	char prefix[4096], name[4200];
	unsigned n, m;
	snprintf(prefix, sizeof(prefix), "%s_untiled", base);
	snprintf(name, sizeof(name), "%s-0", prefix);
	int st = orc_read_header(name, &n, &m);
	if (st) return st;
	unsigned *s = malloc(4 * (size_t) m + 4), *d = malloc(4 * (size_t) m + 4);
	unsigned *deg = malloc(4 * (size_t) n + 4), *rs = malloc(4 * (size_t) n + 4);
	unsigned *map = malloc(4 * (size_t) n + 4);
	if (!s || !d || !deg || !rs || !map) { st = ORC_ENOMEM; goto out; }
	if ((st = orc_read_split(prefix, m, s, d, 0))) goto out;
	snprintf(name, sizeof(name), "%s-nneibor", prefix);
	if ((st = orc_read_lines(name, deg, n))) goto out;
	unsigned acc = 0;
	for (unsigned v = 0; v < n; ++v) { rs[v] = acc; acc += deg[v]; }
	if ((st = orc_vertex_remap_map(n, rs, deg, d, map))) goto out;
	for (unsigned i = 0; i < m; ++i) { s[i] = map[s[i]]; d[i] = map[d[i]]; }
	snprintf(name, sizeof(name), "%s_reorder", base);
	st = orc_write_edge_list(name, n, m, s, d, NULL);
out:
	free(s); free(d); free(deg); free(rs); free(map);
	return st;
}

/* ------------------------------------------------------------------------ */
/* The hybrid BFS (graph_prepare and the steps it calls)                    */
/* ------------------------------------------------------------------------ */

typedef struct orc_graph {
	unsigned n, m, w, s, side;
	const unsigned *vertices; /* CSR row starts (bfs.cpp:1108-1113) */
	const unsigned *degrees;  /* out-degrees (_untiled-nneibor) */
	const unsigned *edges;    /* CSR destinations */
	const unsigned *heads;    /* col-major COO sources */
	const unsigned *tails;    /* col-major COO destinations */
	const unsigned *tile_offsets;
	const unsigned *tile_sizes;
} orc_graph;

/* to_dense (apps/bfs_serial/bfs.cpp:42-56; bfs_simd :54-88). */
static void to_dense(const orc_graph *g, int *mask, int *active_side, const unsigned *queue, unsigned qsize)
{
	memset(mask, 0, sizeof(int) * g->n);
	memset(active_side, 0, sizeof(int) * g->side);
#pragma omp parallel for
	for (unsigned i = 0; i < qsize; ++i) {
		unsigned v = queue[i];
		mask[v] = 1;
		active_side[v / g->w] = 1;
	}
}

/* update_dense (apps/bfs_serial/bfs.cpp:58-106; bfs_simd :91-179). */
static void update_dense(const orc_graph *g, unsigned *out_fsize, unsigned long long *out_deg,
		int *mask, int *updating, int *active_side, int *updating_side)
{
	unsigned long long fsize = 0, odeg = 0;
#pragma omp parallel for reduction(+: fsize, odeg)
	for (unsigned side_id = 0; side_id < g->side; ++side_id) {
		unsigned lo = side_id * g->w;
		unsigned hi = (side_id != g->side - 1) ? lo + g->w : g->n;
		if (!updating_side[side_id]) {
			active_side[side_id] = 0;
			memset(mask + lo, 0, sizeof(int) * (hi - lo));
			continue;
		}
		updating_side[side_id] = 0;
		active_side[side_id] = 1;
		for (unsigned v = lo; v < hi; ++v) {
			if (updating[v] == 1) {
				updating[v] = 0;
				mask[v] = 1;
				fsize++;
				odeg += g->degrees[v];
			} else {
				mask[v] = 0;
			}
		}
	}
	*out_fsize = (unsigned) fsize;
	*out_deg = odeg;
}

/* bfs_kernel_dense over one tile's edges (apps/bfs_serial/bfs.cpp:107-134;
 * the 16-lane form is apps/bfs_simd/bfs.cpp:181-245). */
static void dense_tile(const orc_graph *g, unsigned lo, unsigned hi, const int *mask, int *updating,
		unsigned *parents, int *cost, int *updating_side)
{
	for (unsigned e = lo; e < hi; ++e) {
		unsigned head = g->heads[e];
		if (mask[head] == 0) continue;
		unsigned end = g->tails[e];
		if (parents[end] == UNVISITED) {
			cost[end] = cost[head] + 1;
			updating[end] = 1;
			updating_side[end / g->w] = 1;
			parents[end] = head;
		}
	}
}

/* scheduler_dense: one stripe, dynamic,1 over its columns, skipping empty
 * tiles and tiles whose source row has no frontier vertex
 * (apps/bfs_serial/bfs.cpp:135-183; bfs_simd :246-330). */
static void scheduler_dense(const orc_graph *g, unsigned start_row, unsigned step, const int *mask,
		int *updating, unsigned *parents, int *cost, const int *active_side, int *updating_side)
{
	size_t start_tile = (size_t) start_row * g->side;
	size_t end_tile = start_tile + (size_t) step * g->side;
	if (step == 0) return;
#pragma omp parallel for schedule(dynamic, 1)
	for (long long ti = (long long) start_tile; ti < (long long) end_tile; ti += step) {
		size_t bound = (size_t) ti + step;
		for (size_t t = (size_t) ti; t < bound; ++t) {
			unsigned row = (unsigned) ((t - start_tile) % step) + start_row;
			if (g->tile_sizes[t] == 0 || !active_side[row]) continue;
			dense_tile(g, g->tile_offsets[t], g->tile_offsets[t] + g->tile_sizes[t], mask, updating,
					parents, cost, updating_side);
		}
	}
}

/* BFS_dense: stripes of S rows, then the tail stripe (bfs_simd :331-388). */
static void bfs_dense(const orc_graph *g, const int *mask, int *updating, unsigned *parents, int *cost,
		const int *active_side, int *updating_side)
{
	unsigned rem = g->side % g->s;
	unsigned bound = g->side - rem;
	unsigned side_id;
	for (side_id = 0; side_id < bound; side_id += g->s)
		scheduler_dense(g, side_id, g->s, mask, updating, parents, cost, active_side, updating_side);
	if (rem > 0)
		scheduler_dense(g, side_id, rem, mask, updating, parents, cost, active_side, updating_side);
}

/* to_sparse: mask -> queue through 4096-vertex blocks: count, serial scan,
 * fill (apps/bfs_simd/bfs.cpp:400-465). */
static unsigned *to_sparse(const orc_graph *g, unsigned fsize, const int *mask)
{
	unsigned *queue = (unsigned *) malloc(sizeof(unsigned) * ((size_t) fsize + 1));
	const unsigned block = 1u << 12;
	unsigned nblocks = (g->n - 1) / block + 1;
	unsigned *counts = (unsigned *) calloc(nblocks, sizeof(unsigned));
#pragma omp parallel for
	for (unsigned b = 0; b < nblocks; ++b) {
		unsigned lo = b * block, hi = (b != nblocks - 1) ? lo + block : g->n;
		for (unsigned v = lo; v < hi; ++v) if (mask[v]) counts[b]++;
	}
	unsigned acc = 0;
	for (unsigned b = 0; b < nblocks; ++b) { unsigned t = counts[b]; counts[b] = acc; acc += t; }
#pragma omp parallel for
	for (unsigned b = 0; b < nblocks; ++b) {
		unsigned base = counts[b];
		unsigned lo = b * block, hi = (b != nblocks - 1) ? lo + block : g->n;
		for (unsigned v = lo; v < hi; ++v) if (mask[v]) queue[base++] = v;
	}
	free(counts);
	return queue;
}

/* update_sparse: cost from the parent, sum of out-degrees (bfs_simd :467-509). */
static unsigned long long update_sparse(const orc_graph *g, const unsigned *queue, unsigned qsize,
		const unsigned *parents, int *cost)
{
	unsigned long long odeg = 0;
#pragma omp parallel for reduction(+: odeg)
	for (unsigned i = 0; i < qsize; ++i) {
		unsigned v = queue[i];
		cost[v] = cost[parents[v]] + 1;
		odeg += g->degrees[v];
	}
	return odeg;
}

/* BFS_kernel_sparse: degree gather, serial exclusive scan, CAS expansion with
 * dynamic chunks, blockwise compaction of the (unsigned)-1 holes, final copy
 * (apps/bfs_simd/bfs.cpp:510-711). Returns the new queue (or NULL) and its size. */
static unsigned *bfs_sparse(const orc_graph *g, const unsigned *queue, unsigned *qsize,
		unsigned *parents, unsigned chunk)
{
	unsigned q = *qsize;
	unsigned *offs = (unsigned *) malloc(sizeof(unsigned) * ((size_t) q + 1));
	unsigned long long total = 0;
#pragma omp parallel for reduction(+: total)
	for (unsigned i = 0; i < q; ++i) {
		offs[i] = g->degrees[queue[i]];
		total += offs[i];
	}
	if (total == 0) { free(offs); *qsize = 0; return NULL; }
	unsigned acc = 0;
	for (unsigned i = 0; i < q; ++i) { unsigned t = offs[i]; offs[i] = acc; acc += t; }
	unsigned new_size = (unsigned) total;
	unsigned *tmp = (unsigned *) malloc(sizeof(unsigned) * (size_t) new_size);
#pragma omp parallel for schedule(dynamic, chunk)
	for (unsigned i = 0; i < q; ++i) {
		unsigned start = queue[i];
		unsigned off = offs[i];
		unsigned deg = g->degrees[start];
		unsigned base = g->vertices[start];
		for (unsigned k = 0; k < deg; ++k) {
			unsigned end = g->edges[base + k];
			if (parents[end] == UNVISITED &&
					__sync_bool_compare_and_swap(parents + end, UNVISITED, start))
				tmp[off + k] = end;
			else
				tmp[off + k] = UNVISITED;
		}
	}
	const unsigned block = 2048;
	unsigned nblocks = (new_size - 1) / block + 1;
	unsigned *counts = (unsigned *) malloc(sizeof(unsigned) * nblocks);
	unsigned long long kept = 0;
#pragma omp parallel for reduction(+: kept)
	for (unsigned b = 0; b < nblocks; ++b) {
		unsigned lo = b * block, hi = (b != nblocks - 1) ? lo + block : new_size;
		unsigned base = lo;
		for (unsigned e = lo; e < hi; ++e) if (tmp[e] != UNVISITED) tmp[base++] = tmp[e];
		counts[b] = base - lo;
		kept += counts[b];
	}
	if (kept == 0) { free(offs); free(tmp); free(counts); *qsize = 0; return NULL; }
	unsigned *out = (unsigned *) malloc(sizeof(unsigned) * (size_t) kept);
	acc = 0;
	for (unsigned b = 0; b < nblocks; ++b) { unsigned t = counts[b]; counts[b] = acc; acc += t; }
#pragma omp parallel for
	for (unsigned b = 0; b < nblocks; ++b) {
		unsigned lo = counts[b];
		unsigned hi = (b != nblocks - 1) ? counts[b + 1] : (unsigned) kept;
		memcpy(out + lo, tmp + (size_t) b * block, sizeof(unsigned) * (hi - lo));
	}
	free(offs); free(tmp); free(counts);
	*qsize = (unsigned) kept;
	return out;
}

/*
 * graph_prepare (apps/bfs_simd/bfs.cpp:753-963): initialise, a first top-down
 * step from the source, then the loop that picks dense when
 * frontier_size + out_degree > E / t_ratio (:832-834) and sparse otherwise,
 * converting queue<->mask on a switch, until the frontier is empty.
 *
 * cost/parents: caller-owned arrays of N.  trace (optional): trace[i] = 1 if
 * step i was dense, 0 if sparse; *num_steps = the number of steps run.
 * *seconds: wall time of the traversal, the reference's timed region (:806-913).
 * num_threads <= 0 keeps the OpenMP default.
 */
int orc_bfs_hybrid(unsigned n, unsigned m, const unsigned *vertices, const unsigned *degrees,
		const unsigned *edges, const unsigned *heads, const unsigned *tails,
		const unsigned *tile_offsets, unsigned w, unsigned s, unsigned source,
		unsigned t_ratio, int num_threads, int *cost, unsigned *parents,
		unsigned char *trace, unsigned trace_cap, unsigned *num_steps, double *seconds)
{
	if (n == 0 || source >= n || w == 0 || s == 0 || t_ratio == 0) return ORC_EARG;
	orc_graph g;
	g.n = n; g.m = m; g.w = w; g.s = s; g.side = side_length_of(n, w);
	g.vertices = vertices; g.degrees = degrees; g.edges = edges;
	g.heads = heads; g.tails = tails; g.tile_offsets = tile_offsets;
	size_t num_tiles = (size_t) g.side * g.side;
	unsigned *sizes = (unsigned *) malloc(sizeof(unsigned) * num_tiles);
	for (size_t t = 0; t < num_tiles; ++t)   /* bfs.cpp:1013-1020 */
		sizes[t] = (t != num_tiles - 1) ? tile_offsets[t + 1] - tile_offsets[t] : m - tile_offsets[t];
	g.tile_sizes = sizes;
	if (num_threads > 0) omp_set_num_threads(num_threads);

	int *mask = (int *) calloc(n, sizeof(int));
	int *updating = (int *) calloc(n, sizeof(int));
	int *active_side = (int *) calloc(g.side, sizeof(int));
	int *updating_side = (int *) calloc(g.side, sizeof(int));
	for (unsigned v = 0; v < n; ++v) { cost[v] = -1; parents[v] = UNVISITED; }
	cost[source] = 0;
	parents[source] = source;

	unsigned steps = 0;
	double t0 = omp_get_wtime();
	unsigned fsize = 1;
	unsigned *frontier = (unsigned *) malloc(sizeof(unsigned));
	frontier[0] = source;
	unsigned *nf = bfs_sparse(&g, frontier, &fsize, parents, 2048);
	free(frontier);
	frontier = nf;
	if (trace && steps < trace_cap) trace[steps] = 0;
	steps++;
	unsigned long long odeg = 0;
	for (unsigned i = 0; i < fsize; ++i) {   /* :821-827 */
		unsigned v = frontier[i];
		cost[v] = cost[parents[v]] + 1;
		odeg += degrees[v];
	}
	int last_dense = 0;
	unsigned long long threshold = m / t_ratio;
	while (1) {
		if ((unsigned long long) fsize + odeg > threshold) {
			if (!last_dense) to_dense(&g, mask, active_side, frontier, fsize);
			bfs_dense(&g, mask, updating, parents, cost, active_side, updating_side);
			last_dense = 1;
		} else {
			if (last_dense) {
				nf = to_sparse(&g, fsize, mask);
				free(frontier);
				frontier = nf;
			}
			nf = bfs_sparse(&g, frontier, &fsize, parents, 2048);
			free(frontier);
			frontier = nf;
			last_dense = 0;
		}
		if (trace && steps < trace_cap) trace[steps] = (unsigned char) last_dense;
		steps++;
		if (last_dense) {
			update_dense(&g, &fsize, &odeg, mask, updating, active_side, updating_side);
			if (fsize == 0) break;
		} else {
			if (fsize == 0) break;
			odeg = update_sparse(&g, frontier, fsize, parents, cost);
		}
	}
	double t1 = omp_get_wtime();
	if (seconds) *seconds = t1 - t0;
	if (num_steps) *num_steps = steps;
	free(frontier); free(mask); free(updating); free(active_side); free(updating_side); free(sizes);
	return ORC_OK;
}

/* Plain serial queue BFS over the CSR: the level definition the hybrid must
 * reproduce (every vertex's level is its hop distance from the source). */
int orc_bfs_levels(unsigned n, const unsigned *vertices, const unsigned *degrees,
		const unsigned *edges, unsigned source, int *cost)
{
	if (source >= n) return ORC_EARG;
	unsigned *q = (unsigned *) malloc(sizeof(unsigned) * (size_t) n);
	for (unsigned v = 0; v < n; ++v) cost[v] = -1;
	unsigned head = 0, tail = 0;
	cost[source] = 0;
	q[tail++] = source;
	while (head < tail) {
		unsigned u = q[head++];
		for (unsigned e = vertices[u]; e < vertices[u] + degrees[u]; ++e) {
			unsigned v = edges[e];
			if (cost[v] < 0) { cost[v] = cost[u] + 1; q[tail++] = v; }
		}
	}
	free(q);
	return ORC_OK;
}

/* Parents form a valid BFS tree for these levels: parent[source] = source,
 * every other reached v has an edge parent[v] -> v with
 * level[parent[v]] == level[v] - 1, unreached vertices have (unsigned)-1.
 * Returns the number of violations (0 = valid). */
unsigned long long orc_check_parents(unsigned n, const unsigned *vertices, const unsigned *degrees,
		const unsigned *edges, unsigned source, const int *cost, const unsigned *parents)
{
	unsigned long long bad = 0;
#pragma omp parallel for reduction(+: bad)
	for (unsigned v = 0; v < n; ++v) {
		if (v == source) { bad += (parents[v] != source || cost[v] != 0); continue; }
		if (cost[v] < 0) { bad += (parents[v] != UNVISITED); continue; }
		unsigned p = parents[v];
		if (p >= n || cost[p] != cost[v] - 1) { bad++; continue; }
		int found = 0;
		for (unsigned e = vertices[p]; e < vertices[p] + degrees[p]; ++e)
			if (edges[e] == v) { found = 1; break; }
		bad += !found;
	}
	return bad;
}

int orc_max_threads(void) { return omp_get_max_threads(); }

/* ------------------------------------------------------------------------ */
/* Betweenness-centrality dependencies of one source                        */
/* ------------------------------------------------------------------------ */

/* The reference's BC() (apps/betweennessCentrality_simd/bc.cpp:1717-2097),
 * restated sequentially.
 *
 * Forward: a level-synchronous BFS from `source` in which every edge u -> v
 * from the current frontier to a vertex not visited before this step adds
 * num_paths[u] to num_paths[v] in unsigned 32-bit arithmetic
 * (BFS_kernel_sparse :572-775 with its CAS loop at :640-648, bfs_kernel_dense
 * :1083-1162); the frontiers of every level are kept (:1753-1905).
 * Inverse path counts: 1.0f / (float)(int)num_paths, 0 where num_paths is 0
 * (:1950-1971, a signed conversion).
 * Reverse: from the deepest frontier down to the source's, each frontier
 * vertex is marked visited and adds its inverse to its dependency
 * (update_visited_sparse_reverse :470-503, update_visited_dense_reverse
 * :927-989), then every in-neighbour of it not yet visited in the reverse
 * sweep adds the vertex's dependency (BFS_kernel_sparse_reverse :795-826,
 * bfs_kernel_dense_reverse :1415-1494, over the reverse graph).
 * Finally dependency = (dependency - inverse) / inverse where the inverse is
 * non-zero, else 0 (:2032-2061).  All of it in float, like the reference.
 *
 * The reference's sparse step appends a vertex to the next frontier when its
 * path count was 0 before the add (:649); a count that wraps to exactly 0 mod
 * 2^32 would append it twice.  This restatement takes every vertex once (the
 * BFS levels), which is the reference's result whenever no count wraps to 0.
 *
 * Outputs: num_paths[n], dependencies[n], cost[n] (levels, -1 unreached) and
 * scale[n] (may be NULL): the same recurrence in double over absolute values,
 * (sum |terms|) / |inverse|, the magnitude that bounds the rounding error of a
 * float evaluation in any summation order. */
int orc_bc_single(unsigned n, const unsigned *vertices, const unsigned *degrees, const unsigned *edges,
		unsigned source, unsigned *num_paths, float *dependencies, int *cost, double *scale)
{
	if (source >= n) return ORC_EARG;
	size_t m = 0;
	for (unsigned v = 0; v < n; ++v) m += degrees[v];
	unsigned *q = (unsigned *) malloc(sizeof(unsigned) * (size_t) n);
	unsigned *lvl_beg = (unsigned *) malloc(sizeof(unsigned) * ((size_t) n + 2));
	unsigned *in_off = (unsigned *) calloc((size_t) n + 1, sizeof(unsigned));
	unsigned *in_src = (unsigned *) malloc(sizeof(unsigned) * (m ? m : 1));
	unsigned *fill = (unsigned *) malloc(sizeof(unsigned) * ((size_t) n + 1));
	float *inv = (float *) malloc(sizeof(float) * (size_t) n);
	double *dabs = (double *) malloc(sizeof(double) * (size_t) n);
	char *vis = (char *) calloc(n, 1);
	if (!q || !lvl_beg || !in_off || !in_src || !fill || !inv || !dabs || !vis) {
		free(q); free(lvl_beg); free(in_off); free(in_src); free(fill); free(inv); free(dabs); free(vis);
		return ORC_ENOMEM;
	}
	/* reverse graph: in-edges grouped by destination, sources in CSR order */
	for (unsigned u = 0; u < n; ++u)
		for (unsigned e = vertices[u]; e < vertices[u] + degrees[u]; ++e) in_off[edges[e] + 1]++;
	for (unsigned v = 0; v < n; ++v) in_off[v + 1] += in_off[v];
	memcpy(fill, in_off, sizeof(unsigned) * ((size_t) n + 1));
	for (unsigned u = 0; u < n; ++u)
		for (unsigned e = vertices[u]; e < vertices[u] + degrees[u]; ++e) in_src[fill[edges[e]]++] = u;

	/* forward: frontiers q[lvl_beg[l] .. lvl_beg[l+1]) */
	for (unsigned v = 0; v < n; ++v) { num_paths[v] = 0; cost[v] = -1; dependencies[v] = 0.0f; dabs[v] = 0.0; }
	unsigned nl = 0, tail = 0;
	num_paths[source] = 1;
	cost[source] = 0;
	q[tail++] = source;
	lvl_beg[0] = 0;
	lvl_beg[1] = tail;
	nl = 1;
	while (lvl_beg[nl] > lvl_beg[nl - 1]) {
		const unsigned b = lvl_beg[nl - 1], e = lvl_beg[nl];
		for (unsigned i = b; i < e; ++i) {
			const unsigned u = q[i];
			for (unsigned k = vertices[u]; k < vertices[u] + degrees[u]; ++k) {
				const unsigned v = edges[k];
				if (cost[v] >= 0 && cost[v] < (int) nl) continue; /* visited before this step */
				if (cost[v] < 0) { cost[v] = (int) nl; q[tail++] = v; }
				num_paths[v] += num_paths[u];
			}
		}
		lvl_beg[++nl] = tail;
	}
	/* inverse path counts (signed conversion, as _mm512_cvtepi32_ps) */
	for (unsigned v = 0; v < n; ++v) inv[v] = num_paths[v] ? 1.0f / (float) (int) num_paths[v] : 0.0f;
	/* reverse sweep: levels nl-2 .. 0 hold the non-empty frontiers */
	for (int l = (int) nl - 2; l >= 0; --l) {
		const unsigned b = lvl_beg[l], e = lvl_beg[l + 1];
		for (unsigned i = b; i < e; ++i) {
			const unsigned v = q[i];
			vis[v] = 1;
			dependencies[v] += inv[v];
			dabs[v] += inv[v] < 0 ? -(double) inv[v] : (double) inv[v];
		}
		for (unsigned i = b; i < e; ++i) {
			const unsigned v = q[i];
			for (unsigned k = in_off[v]; k < in_off[v + 1]; ++k) {
				const unsigned u = in_src[k];
				if (vis[u]) continue;
				dependencies[u] += dependencies[v];
				dabs[u] += dabs[v];
			}
		}
	}
	for (unsigned v = 0; v < n; ++v) {
		if (inv[v] != 0.0f) {
			dependencies[v] = (dependencies[v] - inv[v]) / inv[v];
			if (scale) scale[v] = dabs[v] / (inv[v] < 0 ? -(double) inv[v] : (double) inv[v]);
		} else {
			dependencies[v] = 0.0f;
			if (scale) scale[v] = 0.0;
		}
	}
	free(q); free(lvl_beg); free(in_off); free(in_src); free(fill); free(inv); free(dabs); free(vis);
	return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Synthetic input: seeded R-MAT edge lists                                 */
/* ------------------------------------------------------------------------ */

/* The bench's synthetic graphs, generated on the checker's side so that the
 * CPU baseline and the reference arm never load the product library.  The
 * reference itself reads downloaded KONECT files (README.md:15-24); the
 * definition here is the project's own and must give the same edge list as
 * the product's generator (a CPU test compares their digests):
 *   candidate i: for every bit level l < scale (scale = ceil(log2 N)), a
 *   32-bit draw r from h = mix(seed' ^ mix(i*64 + l)) (low half for even l,
 *   high half for odd l, h refreshed at even l) picks the (u,v) bit pair
 *   (0,0) if r < a*2^32, (0,1) if r < (a+b)*2^32, (1,0) if r < (a+b+c)*2^32,
 *   else (1,1); u or v >= N rejects the candidate, and so does u == v when
 *   self loops are dropped;
 *   with dedup, the first occurrence of a (u,v) pair in candidate order is
 *   kept; candidates are taken in order until exactly m edges are kept;
 *   with the permute flag, ids are relabelled by a Fisher-Yates shuffle
 *   driven by the same mix function (perm[v] = the label of v).
 * mix is splitmix64's finaliser; seed' = mix(seed ^ 0x5851F42D4C957F2D).
 * Flags: 1 = no self loops, 2 = dedup, 4 = permute. */
static inline uint64_t orc_mix64(uint64_t x)
{
	x += 0x9E3779B97F4A7C15ull;
	x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
	x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
	return x ^ (x >> 31);
}

static uint32_t orc_threshold(double p)
{
	if (p <= 0) return 0;
	if (p >= 1) return 0xFFFFFFFFu;
	return (uint32_t) (p * 4294967296.0);
}

#define ORC_NO_KEY 0xFFFFFFFFFFFFFFFFull /* u = v = 2^32-1 never occurs: ids are < N <= 2^32-1 */
#define ORC_DEDUP_PARTS 256u

int orc_gen_rmat(unsigned n, unsigned long long m, double a, double b, double c, unsigned long long seed,
		unsigned flags, unsigned *src, unsigned *dst)
{
	const int no_loops = flags & 1, dedup = (flags & 2) != 0, permute = (flags & 4) != 0;
	if (n == 0 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0 + 1e-12) return ORC_EARG;
	if (n == 1 && no_loops && m > 0) return ORC_EARG;
	if (dedup && m > (unsigned long long) n * (no_loops ? n - 1 : n)) return ORC_EARG;
	unsigned scale = 0;
	while ((1ull << scale) < n) ++scale;
	const uint32_t ta = orc_threshold(a), tab = orc_threshold(a + b), tabc = orc_threshold(a + b + c);
	const uint64_t s0 = orc_mix64(seed ^ 0x5851F42D4C957F2Dull);

	/* Per-partition open-addressing sets of the keys seen (partition = top
	 * bits of mix(key)).  A block draws at most 5/4 of the edges still
	 * missing (+ 4096), so at most 5/4 m + 4096 keys are ever inserted; the
	 * sets hold twice that. */
	const uint64_t max_block = 1ull << 22;
	uint64_t per = 1024;
	while (per < ((m + m / 4 + 4096) / ORC_DEDUP_PARTS) * 2 + 1024) per <<= 1;
	uint64_t *table = NULL;
	uint64_t fill[ORC_DEDUP_PARTS];
	int full = 0;
	memset(fill, 0, sizeof(fill));
	if (dedup) {
		table = (uint64_t *) malloc(sizeof(uint64_t) * per * ORC_DEDUP_PARTS);
		if (!table) return ORC_ENOMEM;
		memset(table, 0xFF, sizeof(uint64_t) * per * ORC_DEDUP_PARTS);
	}
	uint64_t *keys = (uint64_t *) malloc(sizeof(uint64_t) * max_block);
	unsigned char *keep = (unsigned char *) malloc(max_block);
	if (!keys || !keep) { free(table); free(keys); free(keep); return ORC_ENOMEM; }
	uint64_t *out = (uint64_t *) malloc(sizeof(uint64_t) * (m ? m : 1));
	if (!out) { free(table); free(keys); free(keep); return ORC_ENOMEM; }
	unsigned long long kept = 0;
	for (uint64_t base = 0, block = 0; kept < m && !full; base += block) {
		block = (m - kept) + (m - kept) / 4 + 4096;
		if (block > max_block) block = max_block;
		/* draw the block's candidates */
		#pragma omp parallel for schedule(static)
		for (int64_t k = 0; k < (int64_t) block; ++k) {
			const uint64_t i = base + (uint64_t) k;
			uint32_t u = 0, v = 0;
			uint64_t h = 0;
			for (unsigned l = 0; l < scale; ++l) {
				if ((l & 1) == 0) h = orc_mix64(s0 ^ orc_mix64(i * 64 + l));
				const uint32_t r = (l & 1) ? (uint32_t) (h >> 32) : (uint32_t) h;
				const uint32_t bu = r >= tab, bv = (r >= ta && r < tab) || r >= tabc;
				u = (u << 1) | bu;
				v = (v << 1) | bv;
			}
			const int bad = u >= n || v >= n || (no_loops && u == v);
			keys[k] = bad ? ORC_NO_KEY : (((uint64_t) u << 32) | v);
			keep[k] = !bad;
		}
		if (dedup) {
			/* each thread owns the partitions p with p % T == t and walks the
			 * block in candidate order: the first occurrence wins */
			#pragma omp parallel
			{
				const unsigned T = (unsigned) omp_get_num_threads(), t = (unsigned) omp_get_thread_num();
				for (uint64_t k = 0; k < block; ++k) {
					const uint64_t key = keys[k];
					if (key == ORC_NO_KEY) continue;
					const uint64_t hk = orc_mix64(key);
					const unsigned part = (unsigned) (hk >> 56);
					if (part % T != t) continue;
					uint64_t *tb = table + (uint64_t) part * per;
					uint64_t slot = (hk & 0xFFFFFFFFull) & (per - 1);
					for (;;) {
						if (tb[slot] == key) { keep[k] = 0; break; }
						if (tb[slot] == ORC_NO_KEY) {
							if (++fill[part] >= per / 2) { full = 1; keep[k] = 0; break; }
							tb[slot] = key;
							break;
						}
						slot = (slot + 1) & (per - 1);
					}
				}
			}
		}
		for (uint64_t k = 0; k < block && kept < m && !full; ++k)
			if (keep[k]) out[kept++] = keys[k];
	}
	free(keys);
	free(keep);
	free(table);
	if (full) { free(out); return ORC_ENOMEM; } /* a partition's set overflowed (never at these sizes) */

	unsigned *perm = NULL;
	if (permute) {
		perm = (unsigned *) malloc(sizeof(unsigned) * n);
		if (!perm) { free(out); return ORC_ENOMEM; }
		for (unsigned v = 0; v < n; ++v) perm[v] = v;
		uint64_t st = orc_mix64(s0 ^ 0xD1B54A32D192ED03ull);
		for (unsigned v = n - 1; v > 0; --v) {
			st = orc_mix64(st);
			const unsigned j = (unsigned) (((unsigned __int128) st * (uint64_t) (v + 1)) >> 64);
			const unsigned x = perm[v];
			perm[v] = perm[j];
			perm[j] = x;
		}
	}
	#pragma omp parallel for schedule(static)
	for (int64_t i = 0; i < (int64_t) m; ++i) {
		unsigned u = (unsigned) (out[i] >> 32), v = (unsigned) out[i];
		if (perm) { u = perm[u]; v = perm[v]; }
		src[i] = u;
		dst[i] = v;
	}
	free(perm);
	free(out);
	return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* BFS level certificate over an edge list                                  */
/* ------------------------------------------------------------------------ */

/* Checks that cost[] are the BFS distances from `source` in the directed
 * edge list (src[i] -> dst[i]) without running a BFS, so that graphs of
 * billions of edges can be checked in seconds: cost is the distance function
 * exactly when
 *   (1) cost[source] == 0 and no other vertex has cost 0 or below -1;
 *   (2) every edge u -> v with cost[u] >= 0 has 0 <= cost[v] <= cost[u] + 1;
 *   (3) every v != source with cost[v] >= 0 has an edge u -> v with
 *       cost[u] == cost[v] - 1.
 * ((2) bounds every reached cost by the distance along any path from the
 * source; (3) gives every reached vertex a path of exactly cost[v] edges.)
 * Returns the number of violated conditions (0 = the levels are the BFS
 * levels).  OpenMP over the edges and the vertices. */
unsigned long long orc_check_levels(unsigned n, unsigned long long m, const unsigned *src, const unsigned *dst,
		unsigned source, const int *cost)
{
	if (source >= n) return 1;
	unsigned long long bad = 0;
	unsigned char *has_parent = (unsigned char *) calloc(n ? n : 1, 1);
	if (!has_parent) return 1;
	if (cost[source] != 0) bad++;
	#pragma omp parallel for schedule(static) reduction(+:bad)
	for (int64_t v = 0; v < (int64_t) n; ++v)
		if ((unsigned) v != source && (cost[v] == 0 || cost[v] < -1)) bad++;
	#pragma omp parallel for schedule(static) reduction(+:bad)
	for (int64_t i = 0; i < (int64_t) m; ++i) {
		const unsigned u = src[i], v = dst[i];
		if (u >= n || v >= n) { bad++; continue; }
		const int cu = cost[u], cv = cost[v];
		if (cu < 0) continue;
		if (cv < 0 || cv > cu + 1) bad++;
		else if (cv == cu + 1) has_parent[v] = 1;  /* a benign race: every writer stores 1 */
	}
	#pragma omp parallel for schedule(static) reduction(+:bad)
	for (int64_t v = 0; v < (int64_t) n; ++v)
		if ((unsigned) v != source && cost[v] > 0 && !has_parent[v]) bad++;
	free(has_parent);
	return bad;
}
