-- H*psi (growing basis, reference OperatorPsi) and restricted H*psi on seeded random
-- operators and wavefunctions.  Output: dump/<case>_{H,psi,Hpsi,Hpsir}.Quanty via io.put.
dofile("common.lua")

-- nf, nel, n1, n2, n4, n6, complex ("r", "c", "m"), ndet, restriction
cases = {
  {name="c10",  nf=10,  nel=4,  n1=0, n2=12, n4=20,  n6=0, kind="r", ndet=30},
  {name="c16",  nf=16,  nel=8,  n1=0, n2=40, n4=80,  n6=0, kind="c", ndet=60},
  {name="m16",  nf=16,  nel=8,  n1=2, n2=30, n4=60,  n6=4, kind="m", ndet=50},
  {name="c26",  nf=26,  nel=18, n1=0, n2=60, n4=100, n6=0, kind="c", ndet=100},
  {name="c64",  nf=64,  nel=20, n1=0, n2=60, n4=60,  n6=2, kind="c", ndet=80},
  {name="c70",  nf=70,  nel=35, n1=0, n2=60, n4=60,  n6=0, kind="c", ndet=80},
  {name="r100", nf=100, nel=50, n1=2, n2=60, n4=60,  n6=0, kind="r", ndet=80},
  {name="c128", nf=128, nel=30, n1=0, n2=60, n4=60,  n6=2, kind="c", ndet=60},
}

function rand_value(kind)
  local re = 2 * pm_uniform() - 1
  if kind == "r" then return re end
  local im = 2 * pm_uniform() - 1
  return re + I * im
end

-- pick k distinct orbitals in 0..nf-1
function distinct(nf, k)
  local out, used = {}, {}
  while #out < k do
    local v = pm_int(nf)
    if not used[v] then used[v] = true; out[#out + 1] = v end
  end
  return out
end

-- orbitals are chosen near an occupied/empty boundary often enough that terms apply
function make_operator(c)
  local terms = {}
  terms[#terms + 1] = {0.25}
  local function val(len)
    if c.kind == "m" then
      if len == 2 then return rand_value("c") else return rand_value("r") end
    end
    return rand_value(c.kind)
  end
  for t = 1, c.n1 do
    local o = distinct(c.nf, 1)
    if t % 2 == 1 then terms[#terms + 1] = {o[1], val(1)} else terms[#terms + 1] = {-o[1], val(1)} end
  end
  for t = 1, c.n2 do
    local o = distinct(c.nf, 2)
    terms[#terms + 1] = {o[1], -o[2], val(2)}
  end
  for t = 1, c.n4 do
    local o = distinct(c.nf, 4)
    terms[#terms + 1] = {o[1], o[2], -o[3], -o[4], val(4)}
  end
  for t = 1, c.n6 do
    local o = distinct(c.nf, 6)
    terms[#terms + 1] = {o[1], o[2], o[3], -o[4], -o[5], -o[6], val(6)}
  end
  return NewOperator(c.nf, 0, terms)
end

function make_psi(c)
  local all = {}
  for i = 0, c.nf - 1 do all[#all + 1] = i end
  local list, seen = {}, {}
  while #list < c.ndet do
    local d = random_det(c.nf, {{all, c.nel}})
    if not seen[d] then
      seen[d] = true
      local v = rand_value(c.kind == "r" and "r" or "c")
      list[#list + 1] = {d, v}
    end
  end
  return NewWavefunction(c.nf, 0, list)
end

for ic, c in ipairs(cases) do
  pm_seed(1000 + 7 * ic)
  local H = make_operator(c)
  local psi = make_psi(c)
  local Hpsi = H * psi
  _G[c.name .. "_H"] = H
  _G[c.name .. "_psi"] = psi
  _G[c.name .. "_Hpsi"] = Hpsi
  io.put("dump", c.name .. "_H")
  io.put("dump", c.name .. "_psi")
  io.put("dump", c.name .. "_Hpsi")
  -- restriction: the first half of the orbitals holds between (nel/2 - 1) and (nel/2 + 1) electrons
  local mask = {}
  for i = 1, c.nf do mask[i] = (i <= c.nf / 2) and "1" or "0" end
  local lo = math.floor(c.nel / 2) - 1
  local hi = math.floor(c.nel / 2) + 1
  if lo < 0 then lo = 0 end
  H.Restrictions = {c.nf, 0, {table.concat(mask), lo, hi}}
  local Hpsir = H * psi
  _G[c.name .. "_Hpsir"] = Hpsir
  io.put("dump", c.name .. "_Hpsir")
  dump_reals("dump/" .. c.name .. "_restriction.txt", {lo, hi})
end
print("hpsi_cases done")
