"""The closed form of gpu/bvh.js's swap-with-the-end partition that the GPU BVH build uses (csrc/vt_bvh_gpu.cu),
restated step by step and checked against the loop itself on random ranges:
- the single-group form (run_task): with m0 = s + (left slots), the k-th right slot of [s, m0) trades places with the
  k-th left slot of [m0, e) counted from the top (q_k) and moves to q_{k-1} - 1 (q_0 = e); a right slot x of [m0, e)
  moves to x - 1, except x = m0, which moves to q_K - 1;
- the chunked form of the top levels (big_part_top, big_part_bottom): a chunk's ranks start after the left slots of
  the chunks above it and the right slots of the chunks below it, so only per-chunk left counts cross chunks."""
import random


def swap_loop(order, s, e, left):
    o = list(order)
    i, j = s, e - 1
    while i <= j:
        t = o[i]
        if left(t):
            i += 1
        else:
            o[i] = o[j]
            o[j] = t
            j -= 1
    return o, i


def chunked(order, s, e, left, chunk):
    o = list(order)
    scratch = list(o)
    qpos = [None] * len(o)
    chunks = [(a, min(e, a + chunk)) for a in range(s, e, chunk)]
    nleft = [sum(1 for p in range(a, b) if left(o[p])) for a, b in chunks]
    m0 = s + sum(nleft)
    k_at_m0 = None
    for c, (a, b) in enumerate(chunks):          # pass 1: [m0, e) from the top
        k = sum(nleft[c + 1:])
        for x in range(b - 1, max(a, m0) - 1, -1):
            if left(o[x]):
                qpos[s + k] = x
                k += 1
            elif x > m0:
                scratch[x - 1] = o[x]
        if a <= m0 < b:
            k_at_m0 = k
    for c, (a, b) in enumerate(chunks):          # pass 2: [s, m0) from the bottom, and the slot at m0
        if a <= m0 < b and not left(o[m0]):
            scratch[(qpos[s + k_at_m0 - 1] if k_at_m0 else e) - 1] = o[m0]
        k = sum((chunks[j][1] - chunks[j][0]) - nleft[j] for j in range(c))
        for p in range(a, min(b, m0)):
            t = o[p]
            if left(t):
                scratch[p] = t
            else:
                k += 1
                scratch[(e if k == 1 else qpos[s + k - 2]) - 1] = t
                scratch[p] = o[qpos[s + k - 1]]
    o[s:e] = scratch[s:e]
    return o, m0


def test_chunked_closed_form_matches_swap_loop():
    rng = random.Random(1)
    for _ in range(4000):
        n = rng.randint(1, 200)
        s = rng.randint(0, 4)
        e = s + n
        order = list(range(e + rng.randint(0, 4)))
        rng.shuffle(order)
        p_left = rng.random()
        flags = {t: rng.random() < p_left for t in order}
        chunk = rng.choice([1, 2, 3, 7, 16, 64, 1000])
        want, m_want = swap_loop(order, s, e, flags.__getitem__)
        got, m_got = chunked(order, s, e, flags.__getitem__, chunk)
        assert got == want and m_got == m_want, (n, chunk)
