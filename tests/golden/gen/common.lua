-- Shared helpers for the fixture generators (run by the reference Quanty binary).
-- Deterministic: no math.random; a Park-Miller generator x <- 16807 x mod (2^31-1).
Verbosity(0)
pm_state = 20240601
function pm_seed(s) pm_state = s end
function pm_next()
  pm_state = (16807 * pm_state) % 2147483647
  return pm_state
end
-- uniform in [0,1)
function pm_uniform() return (pm_next() - 1) / 2147483646 end
function pm_int(n) return math.floor(pm_uniform() * n) end   -- 0..n-1

-- write a list of real numbers, one per line, full precision
function dump_reals(fname, t)
  local f = io.open(fname, "w")
  for i = 1, #t do f:write(string.format("%.17g\n", t[i])) end
  f:close()
end
-- write a list of (possibly complex) numbers as "re im" lines
function dump_complex(fname, t)
  local f = io.open(fname, "w")
  for i = 1, #t do
    local z = t[i]
    if type(z) == "number" then
      f:write(string.format("%.17g 0\n", z))
    else
      f:write(string.format("%.17g %.17g\n", Complex.Re(z), Complex.Im(z)))
    end
  end
  f:close()
end
-- write a tridiagonal table {a, b} as returned by CreateSpectra
function dump_tri(fname, G)
  local f = io.open(fname, "w")
  local a, b = G[1], G[2]
  f:write(string.format("%d %d\n", #a, #b))
  for i = 1, #a do f:write(string.format("%.17g\n", a[i])) end
  for i = 1, #b do f:write(string.format("%.17g\n", b[i])) end
  f:close()
end
-- random determinant string with nel electrons among the orbitals listed in idx (0-based)
function random_det(nf, occ_sets)
  local bits = {}
  for i = 1, nf do bits[i] = "0" end
  for _, s in ipairs(occ_sets) do
    local idx, nel = s[1], s[2]
    local pool = {}
    for _, v in ipairs(idx) do pool[#pool + 1] = v end
    for k = 1, nel do
      local j = pm_int(#pool) + 1
      bits[pool[j] + 1] = "1"
      table.remove(pool, j)
    end
  end
  return table.concat(bits)
end
