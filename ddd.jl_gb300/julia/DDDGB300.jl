# DDDGB300.jl — Julia binding of libddd_gb300.so (include/ddd_gb300.h) for DDD.jl.
#
# Drop-in for the O(N^2) hot path: calcSegSegForce / calcSegSegForce! /
# calc_σTilde / calc_σTilde! keep DDD.jl's signatures and array layouts; the
# network's own arrays are passed to the library without copies.  Select it
# with the existing DislocationParameters field parGPU (src/Type/DislocationType.jl:254):
# one line at the top of each replaced function, e.g. in calcSegSegForce
# (src/Processing/DislocationForces.jl:470):
#     dlnParams.parGPU && return DDDGB300.calcSegSegForceGPU(dlnParams, matParams, network, idx)
#
# Julia is not installed in the environment this library was built in, so this
# file has not been executed there; the C ABI it binds is exercised by the
# Python mirror (ddd.jl_gb300/__init__.py) and its tests.
module DDDGB300

using Statistics: mean

export calcSegSegForceGPU, calcSegSegForceGPU!, calc_σTildeGPU, calc_σTildeGPU!
export calcSelfForceGPU, calcSelfForceGPU!, calcSegForceGPU, calcSegForceGPU!
export Surrogate, loadSurrogate, quadratureFarField, calcSegSegForceSurrogateGPU
export dlnMobilityGPU, dlnMobilityGPU!, detectCollisionGPU, minimumDistanceGPU, calc_uTildeGPU, calc_uTildeGPU!
export setPartialLimitGPU, partialLimitGPU, setModeGPU, modeGPU

const libddd = joinpath(@__DIR__, "..", "libddd_gb300.so")

struct DDDConsts
    aSq::Float64
    mu4pi::Float64
    mu8pi::Float64
    mu4pinu::Float64
    nuMu4pinu::Float64
end

const CTX = Ref{Ptr{Cvoid}}(C_NULL)

function context()
    if CTX[] == C_NULL
        p = ccall((:ddd_create, libddd), Ptr{Cvoid}, (Cint,), 0)
        p == C_NULL && error("ddd_create: " * unsafe_string(ccall((:ddd_last_error, libddd), Cstring, (Ptr{Cvoid},), C_NULL)))
        CTX[] = p
        atexit(() -> ccall((:ddd_destroy, libddd), Cvoid, (Ptr{Cvoid},), CTX[]))
    end
    return CTX[]
end

consts(dlnParams, matParams) =
    DDDConsts(dlnParams.coreRadSq, matParams.μ4π, matParams.μ8π, matParams.μ4πν, matParams.νμ4πν)

function check(rc)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:ddd_last_error, libddd), Cstring, (Ptr{Cvoid},), context()))
    rc == -2 && throw(BoundsError(msg))
    (rc == -1 || rc == -3) && throw(ArgumentError(msg))
    error("libddd_gb300 error $rc: $msg")
end

idxvec(idx) = isnothing(idx) ? Int64[] : collect(Int64, idx)

# Device memory for the all-pairs partial sums (bytes; 0 = the 16 GiB
# default).  Networks whose tile pairs need more run in bands of tile columns
# through a buffer of this size (same forces to rounding, deterministic).
setPartialLimitGPU(bytes::Integer) =
    check(ccall((:ddd_set_partial_limit, libddd), Cint, (Ptr{Cvoid}, Int64), context(), bytes))
partialLimitGPU() = ccall((:ddd_get_partial_limit, libddd), Int64, (Ptr{Cvoid},), context())

# Arithmetic of the context's kernels (ddd_set_mode): 0 = strict FP64, the
# reference's formulas and rounding (default); 4 = the fast FP64 form (same
# formulas, fewer FP64 instructions, within the strict form's parity bound);
# 1 = FP64 with FMA contraction; 2 = df64; 3 = f32c.
setModeGPU(mode::Integer) = check(ccall((:ddd_set_mode, libddd), Cint, (Ptr{Cvoid}, Cint), context(), mode))
modeGPU() = ccall((:ddd_get_mode, libddd), Cint, (Ptr{Cvoid},), context())

# calcSegSegForce (src/Processing/DislocationForces.jl:470-561)
function calcSegSegForceGPU(dlnParams, matParams, network, idx = nothing)
    numSeg = network.numSeg[1]
    iv = idxvec(idx)
    n = isnothing(idx) ? numSeg : length(iv)
    out = zeros(3, 2, n)
    k = Ref(consts(dlnParams, matParams))
    coord, bVec, segIdx, extSeg = network.coord, network.bVec, network.segIdx, network.extSeg
    GC.@preserve coord bVec segIdx extSeg iv out begin
        rc = ccall((:ddd_segseg_force, libddd), Cint,
            (Ptr{Cvoid}, Ref{DDDConsts}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Int64}, Int64,
             Ptr{Bool}, Int64, Ptr{Int64}, Int64, Ptr{Float64}, Ptr{Cvoid}),
            context(), k, coord, size(coord, 2), bVec, size(bVec, 2), segIdx, size(segIdx, 1),
            extSeg, numSeg, isnothing(idx) ? C_NULL : pointer(iv), length(iv), out, C_NULL)
    end
    check(rc)
    return out
end

# calcSegSegForce! (src/Processing/DislocationForces.jl:576-669)
function calcSegSegForceGPU!(dlnParams, matParams, network, idx = nothing)
    numSeg = network.numSeg[1]
    iv = idxvec(idx)
    k = Ref(consts(dlnParams, matParams))
    coord, bVec, segIdx, extSeg, segForce = network.coord, network.bVec, network.segIdx, network.extSeg, network.segForce
    GC.@preserve coord bVec segIdx extSeg segForce iv begin
        rc = ccall((:ddd_segseg_force_inplace, libddd), Cint,
            (Ptr{Cvoid}, Ref{DDDConsts}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Int64}, Int64,
             Ptr{Bool}, Int64, Ptr{Int64}, Int64, Ptr{Float64}, Int64, Ptr{Cvoid}),
            context(), k, coord, size(coord, 2), bVec, size(bVec, 2), segIdx, size(segIdx, 1),
            extSeg, numSeg, isnothing(idx) ? C_NULL : pointer(iv), length(iv), segForce, size(segForce, 3), C_NULL)
    end
    check(rc)
    return nothing
end

# calc_σTilde! (src/Processing/DislocationFEM.jl:67-84); x0 must be a 3×M array.
function calc_σTildeGPU!(σ, x0, dlnParams, matParams, network, idx = nothing)
    @assert ndims(σ) == ndims(x0) && size(σ, 1) == 6
    @assert size(σ, 2) == size(x0, 2)
    iv = idxvec(idx)
    k = Ref(consts(dlnParams, matParams))
    coord, bVec, segIdx = network.coord, network.bVec, network.segIdx
    xs = convert(Array{Float64}, x0)
    GC.@preserve coord bVec segIdx xs σ iv begin
        rc = ccall((:ddd_sigma_tilde, libddd), Cint,
            (Ptr{Cvoid}, Ref{DDDConsts}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Float64}, Int64,
             Ptr{Int64}, Int64, Int64, Ptr{Int64}, Int64, Ptr{Float64}, Ptr{Cvoid}),
            context(), k, xs, size(xs, 2), coord, size(coord, 2), bVec, size(bVec, 2), segIdx, size(segIdx, 1),
            network.numSeg[1], isnothing(idx) ? C_NULL : pointer(iv), length(iv), σ, C_NULL)
    end
    check(rc)
    return σ
end

# calc_σTilde (src/Processing/DislocationFEM.jl:24-41)
function calc_σTildeGPU(x0, dlnParams, matParams, network, idx = nothing)
    xs = x0 isa Base.Iterators.ProductIterator ? reduce(hcat, [collect(p) for p in x0]) : x0
    numPoints = div(length(xs), 3)
    xs = reshape(convert(Array{Float64}, xs), 3, numPoints)
    σ = zeros(6, numPoints)
    calc_σTildeGPU!(σ, xs, dlnParams, matParams, network, idx)
    return numPoints == 1 ? σ[:, 1] : σ
end

# ---------------------------------------------------------------------------
# Self force and total segment force (DislocationForces.jl:23-72, 320-455).

struct DDDSelfParams
    coreRad::Float64
    coreEnergy::Float64
    nu::Float64
end

selfparams(dlnParams, matParams) = DDDSelfParams(dlnParams.coreRad, dlnParams.coreEnergy, matParams.ν)

# calcSelfForce: (selfForceNode1, selfForceNode2), 3×n each
function calcSelfForceGPU(dlnParams, matParams, network, idx = nothing)
    numSeg = network.numSeg[1]
    iv = idxvec(idx)
    n = isnothing(idx) ? numSeg : length(iv)
    F1, F2 = zeros(3, n), zeros(3, n)
    k, sp = Ref(consts(dlnParams, matParams)), Ref(selfparams(dlnParams, matParams))
    coord, bVec, segIdx, extSeg = network.coord, network.bVec, network.segIdx, network.extSeg
    GC.@preserve coord bVec segIdx extSeg iv F1 F2 begin
        rc = ccall((:ddd_self_force, libddd), Cint,
            (Ptr{Cvoid}, Ref{DDDConsts}, Ref{DDDSelfParams}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Int64},
             Int64, Ptr{Bool}, Int64, Ptr{Int64}, Int64, Ptr{Float64}, Ptr{Float64}),
            context(), k, sp, coord, size(coord, 2), bVec, size(bVec, 2), segIdx, size(segIdx, 1), extSeg, numSeg,
            isnothing(idx) ? C_NULL : pointer(iv), length(iv), F1, F2)
    end
    check(rc)
    return F1, F2
end

# calcSelfForce!
function calcSelfForceGPU!(dlnParams, matParams, network, idx = nothing)
    numSeg = network.numSeg[1]
    iv = idxvec(idx)
    k, sp = Ref(consts(dlnParams, matParams)), Ref(selfparams(dlnParams, matParams))
    coord, bVec, segIdx, extSeg, segForce = network.coord, network.bVec, network.segIdx, network.extSeg, network.segForce
    GC.@preserve coord bVec segIdx extSeg segForce iv begin
        rc = ccall((:ddd_self_force_inplace, libddd), Cint,
            (Ptr{Cvoid}, Ref{DDDConsts}, Ref{DDDSelfParams}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Int64},
             Int64, Ptr{Bool}, Int64, Ptr{Int64}, Int64, Ptr{Float64}, Int64),
            context(), k, sp, coord, size(coord, 2), bVec, size(bVec, 2), segIdx, size(segIdx, 1), extSeg, numSeg,
            isnothing(idx) ? C_NULL : pointer(iv), length(iv), segForce, size(segForce, 3))
    end
    check(rc)
    return nothing
end

# calcSegForce with the FE stress at the segment midpoints given as data:
# σHat (6×n: xx, yy, zz, xy, xz, yz) = calc_σHat(mesh, forceDisplacement, midpoint)
# for each entry, or `nothing` for no PK term.
function calcSegForceGPU(dlnParams, matParams, σHat, network, idx = nothing)
    numSeg = network.numSeg[1]
    iv = idxvec(idx)
    n = isnothing(idx) ? numSeg : length(iv)
    out = zeros(3, 2, n)
    sh = isnothing(σHat) ? Float64[] : convert(Array{Float64}, σHat)
    k, sp = Ref(consts(dlnParams, matParams)), Ref(selfparams(dlnParams, matParams))
    coord, bVec, segIdx, extSeg = network.coord, network.bVec, network.segIdx, network.extSeg
    GC.@preserve coord bVec segIdx extSeg iv out sh begin
        rc = ccall((:ddd_seg_force, libddd), Cint,
            (Ptr{Cvoid}, Ref{DDDConsts}, Ref{DDDSelfParams}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Int64},
             Int64, Ptr{Bool}, Int64, Ptr{Float64}, Ptr{Int64}, Int64, Ptr{Float64}, Ptr{Cvoid}),
            context(), k, sp, coord, size(coord, 2), bVec, size(bVec, 2), segIdx, size(segIdx, 1), extSeg, numSeg,
            isnothing(σHat) ? C_NULL : pointer(sh), isnothing(idx) ? C_NULL : pointer(iv), length(iv), out, C_NULL)
    end
    check(rc)
    return out
end

# calcSegForce!
function calcSegForceGPU!(dlnParams, matParams, σHat, network, idx = nothing)
    numSeg = network.numSeg[1]
    iv = idxvec(idx)
    sh = isnothing(σHat) ? Float64[] : convert(Array{Float64}, σHat)
    k, sp = Ref(consts(dlnParams, matParams)), Ref(selfparams(dlnParams, matParams))
    coord, bVec, segIdx, extSeg, segForce = network.coord, network.bVec, network.segIdx, network.extSeg, network.segForce
    GC.@preserve coord bVec segIdx extSeg segForce iv sh begin
        rc = ccall((:ddd_seg_force_inplace, libddd), Cint,
            (Ptr{Cvoid}, Ref{DDDConsts}, Ref{DDDSelfParams}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Int64},
             Int64, Ptr{Bool}, Int64, Ptr{Float64}, Ptr{Int64}, Int64, Ptr{Float64}, Int64, Ptr{Cvoid}),
            context(), k, sp, coord, size(coord, 2), bVec, size(bVec, 2), segIdx, size(segIdx, 1), extSeg, numSeg,
            isnothing(σHat) ? C_NULL : pointer(sh), isnothing(idx) ? C_NULL : pointer(iv), length(iv), segForce,
            size(segForce, 3), C_NULL)
    end
    check(rc)
    return nothing
end

# ---------------------------------------------------------------------------
# BCC mobility (DislocationMobility.jl:16-178 and dlnMobility! :186-): node
# forces from network.segForce and node velocities from the 3×3 drag solve.

struct DDDMobParams
    sigmaPN::Float64
    edgeDrag::Float64
    screwDrag::Float64
    climbDrag::Float64
    lineDrag::Float64
end

function mobparams(dlnParams, matParams)
    d = dlnParams.dragCoeffs
    return DDDMobParams(matParams.σPN, d.edge, d.screw, d.climb, d.line)
end

# dlnMobility: (nodeForce, nodeVel), 3×n each
function dlnMobilityGPU(dlnParams, matParams, network, idx = nothing)
    numNode = network.numNode[1]
    iv = idxvec(idx)
    n = isnothing(idx) ? numNode : length(iv)
    F, V = zeros(3, n), zeros(3, n)
    mp = Ref(mobparams(dlnParams, matParams))
    coord, bVec, links, conn, segForce = network.coord, network.bVec, network.links, network.connectivity,
                                         network.segForce
    GC.@preserve coord bVec links conn segForce iv F V begin
        rc = ccall((:ddd_mobility_bcc, libddd), Cint,
            (Ptr{Cvoid}, Ref{DDDMobParams}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Int64}, Int64, Ptr{Int64},
             Int64, Int64, Ptr{Float64}, Int64, Int64, Ptr{Int64}, Int64, Ptr{Float64}, Ptr{Float64}),
            context(), mp, coord, size(coord, 2), bVec, size(bVec, 2), links, size(links, 2), conn, size(conn, 1),
            size(conn, 2), segForce, size(segForce, 3), numNode, isnothing(idx) ? C_NULL : pointer(iv), length(iv),
            F, V)
    end
    check(rc)
    return F, V
end

# dlnMobility!: writes the nodes' columns of network.nodeForce and network.nodeVel
function dlnMobilityGPU!(dlnParams, matParams, network, idx = nothing)
    numNode = network.numNode[1]
    iv = idxvec(idx)
    mp = Ref(mobparams(dlnParams, matParams))
    coord, bVec, links, conn, segForce = network.coord, network.bVec, network.links, network.connectivity,
                                         network.segForce
    nodeForce, nodeVel = network.nodeForce, network.nodeVel
    GC.@preserve coord bVec links conn segForce nodeForce nodeVel iv begin
        rc = ccall((:ddd_mobility_bcc_inplace, libddd), Cint,
            (Ptr{Cvoid}, Ref{DDDMobParams}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Int64}, Int64, Ptr{Int64},
             Int64, Int64, Ptr{Float64}, Int64, Int64, Ptr{Int64}, Int64, Ptr{Float64}, Ptr{Float64}, Int64),
            context(), mp, coord, size(coord, 2), bVec, size(bVec, 2), links, size(links, 2), conn, size(conn, 1),
            size(conn, 2), segForce, size(segForce, 3), numNode, isnothing(idx) ? C_NULL : pointer(iv), length(iv),
            nodeForce, nodeVel, size(nodeForce, 2))
    end
    check(rc)
    return nothing
end

# ---------------------------------------------------------------------------
# Collision detection (DislocationTopologyCollision.jl:1-221) and
# minimumDistance (Misc.jl:314-367).

struct DDDCollision
    collision::Int32
    type::Int32
    n1s1::Int64
    n2s1::Int64
    n1s2::Int64
    n2s2::Int64
    s1::Int64
    s2::Int64
    L1::Float64
    L2::Float64
    pairDistSq::Float64
    pairL1::Float64
    pairL2::Float64
end

# detectCollision: the reference's 10-tuple (network.label is Int32-backed).
function detectCollisionGPU(dlnParams, network, skipSegs = Vector{Tuple{Int, Int}}())
    r = Ref{DDDCollision}()
    sk = collect(Tuple{Int, Int}, skipSegs)
    coord, nodeVel, label, links, bVec, conn = network.coord, network.nodeVel, network.label, network.links,
                                               network.bVec, network.connectivity
    GC.@preserve coord nodeVel label links bVec conn sk begin
        rc = ccall((:ddd_detect_collision, libddd), Cint,
            (Ptr{Cvoid}, Float64, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Cvoid}, Int64, Ptr{Int64}, Int64,
             Ptr{Float64}, Int64, Ptr{Int64}, Int64, Int64, Int64, Int64, Ptr{Cvoid}, Int64, Ref{DDDCollision}),
            context(), dlnParams.collisionDistSq, coord, size(coord, 2), nodeVel, size(nodeVel, 2), pointer(label),
            length(label), links, size(links, 2), bVec, size(bVec, 2), conn, size(conn, 1), size(conn, 2),
            network.numNode[1], network.numSeg[1], pointer(sk), length(sk), r)
    end
    check(rc)
    c = r[]
    return c.collision == 1, (:null, :hinge, :twoLine)[c.type + 1], c.n1s1, c.n2s1, c.n1s2, c.n2s2, c.s1, c.s2,
           c.L1, c.L2
end

# minimumDistance for one pair of segments.
function minimumDistanceGPU(x0, x1, y0, y1, vx0, vx1, vy0, vy1)
    pts = Float64[x0; x1; y0; y1; vx0; vx1; vy0; vy1]
    out = zeros(4)
    GC.@preserve pts out begin
        rc = ccall((:ddd_minimum_distance, libddd), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int64, Ptr{Float64}),
                   context(), pts, 1, out)
    end
    check(rc)
    return out[1], out[2], out[3], out[4]
end

# ---------------------------------------------------------------------------
# calc_uTilde / calc_uTilde! (DislocationFEM.jl:354-632): the mesh enters as
# data (closure point, bounding box, face normals and midpoints, the normals
# used for projections).

struct DDDUMesh
    C::NTuple{3, Float64}
    lo::NTuple{3, Float64}
    hi::NTuple{3, Float64}
    tol::Float64
    faceNorm::Ptr{Float64}
    faceMidPt::Ptr{Float64}
    numFaces::Int64
    normals::Ptr{Float64}
    numNormals::Int64
end

function _u_tilde!(uTilde, uDofs, mesh, boundaries, matParams, network)
    C = Tuple(mean(mesh.vertices.vertices))
    V = reduce(hcat, mesh.vertices.vertices)
    lo, hi = Tuple(minimum(V, dims = 2)), Tuple(maximum(V, dims = 2))
    faceNorm, faceMidPt = Matrix{Float64}(mesh.faceNorm), Matrix{Float64}(mesh.faceMidPt)
    normals = mesh isa ..AbstractRegularCuboidMesh ? faceNorm[:, 1:2:5] : faceNorm  # DDD's mesh type (parent module)
    points = Matrix{Float64}(mesh.coord[:, boundaries.uGammaDln])
    coord, label, links, bVec = network.coord, network.label, network.links, network.bVec
    dofs = uDofs === nothing ? C_NULL : convert(Vector{Int64}, uDofs)
    GC.@preserve faceNorm faceMidPt normals points coord label links bVec dofs uTilde begin
        m = Ref(DDDUMesh(C, lo, hi, 0.0, pointer(faceNorm), pointer(faceMidPt), size(faceNorm, 2), pointer(normals),
                         size(normals, 2)))
        rc = ccall((:ddd_u_tilde, libddd), Cint,
            (Ptr{Cvoid}, Float64, Float64, Ref{DDDUMesh}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Cvoid},
             Int64, Ptr{Int64}, Int64, Ptr{Float64}, Int64, Int64, Int64, Ptr{Cvoid}, Ptr{Float64}, Int64),
            context(), matParams.omνInv8π, matParams.om2νomνInv8π, m, points, size(points, 2), coord, size(coord, 2),
            pointer(label), length(label), links, size(links, 2), bVec, size(bVec, 2), network.numNode[1],
            network.numSeg[1], dofs === C_NULL ? C_NULL : pointer(dofs), uTilde, length(uTilde))
    end
    check(rc)
    return uTilde
end

# calc_uTilde: point-major vector over boundaries.uGammaDln
calc_uTildeGPU(mesh, boundaries, matParams, network) =
    _u_tilde!(zeros(3 * length(boundaries.uGammaDln)), nothing, mesh, boundaries, matParams, network)

# calc_uTilde!: zero forceDisplacement.uTilde, add through boundaries.uDofsDln
function calc_uTildeGPU!(forceDisplacement, mesh, boundaries, matParams, network)
    u = zeros(length(forceDisplacement.uTilde))
    _u_tilde!(u, boundaries.uDofsDln, mesh, boundaries, matParams, network)
    forceDisplacement.uTilde .= u
    return nothing
end

# ---------------------------------------------------------------------------
# Learned far-field surrogate (no reference counterpart): calcSegSegForce with
# far pairs (R >= kappa max(L_i, L_j)) from a trained network and near pairs
# exact; checkpoints as written by ddd_surrogate_save (e.g. the repository's
# ddd.jl_gb300/data/surrogate_gpu65k_nu028.bin, trained for nu = 0.28).

struct DDDSurOpts
    kappa::Float64
    audit_fraction::Float64
    audit_tol::Float64
    exact_mode::Cint
    far_mode::Cint
    kappa_two::Float64
end

struct DDDSurReport
    pairs_total::Int64
    pairs_near_general::Int64
    pairs_near_parallel::Int64
    tiles_total::Int64
    tiles_near::Int64
    tiles_audit::Int64
    audit_rel_rms::Float64
    audit_rel_max::Float64
    audit_node_rel_rms::Float64
    fallback::Cint
    ms_prep::Float64
    ms_network::Float64
    ms_audit::Float64
    ms_near::Float64
    ms_reduce::Float64
    ms_total::Float64
end

mutable struct Surrogate
    ptr::Ptr{Cvoid}
    kappa::Float64
    nu::Float64
end

function surcheck(s::Surrogate, rc)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:ddd_surrogate_last_error, libddd), Cstring, (Ptr{Cvoid},), s.ptr))
    rc == -2 && throw(BoundsError(msg))
    (rc == -1 || rc == -3) && throw(ArgumentError(msg))
    error("libddd_gb300 surrogate error $rc: $msg")
end

function loadSurrogate(path::AbstractString)
    p = ccall((:ddd_surrogate_create, libddd), Ptr{Cvoid}, (Ptr{Cvoid}, UInt64), context(), 0)
    p == C_NULL && error("ddd_surrogate_create failed")
    s = Surrogate(p, 0.0, 0.0)
    finalizer(x -> ccall((:ddd_surrogate_destroy, libddd), Cvoid, (Ptr{Cvoid},), x.ptr), s)
    kappa, nu, aSq = Ref(0.0), Ref(0.0), Ref(0.0)
    surcheck(s, ccall((:ddd_surrogate_load, libddd), Cint, (Ptr{Cvoid}, Cstring, Ref{Float64}, Ref{Float64},
                                                             Ref{Float64}), p, path, kappa, nu, aSq))
    s.kappa, s.nu = kappa[], nu[]
    return s
end

# A handle without a checkpoint, for far_mode = 2 or 3 (the quadrature reads
# no weights); kappa is the near/far threshold R >= kappa max(L_i, L_j).  The
# 3-point rule (far_mode 3) is at its FP32 noise level (~2e-7 per pair) from
# R = 8 max(L) on, so 10 suffices; the 2-point rule needs 20.
function quadratureFarField(; kappa = 10.0)
    p = ccall((:ddd_surrogate_create, libddd), Ptr{Cvoid}, (Ptr{Cvoid}, UInt64), context(), 0)
    p == C_NULL && error("ddd_surrogate_create failed")
    s = Surrogate(p, kappa, NaN)
    finalizer(x -> ccall((:ddd_surrogate_destroy, libddd), Cvoid, (Ptr{Cvoid},), x.ptr), s)
    return s
end

# exact_mode: 0 = strict FP64 (DDD_MODE_FP64), 4 = fast FP64, 2 = df64, 3 = f32c.
# far_mode: 0 = far pairs through the network; 2 or 3 = Gauss-Legendre
# quadrature with that many points per segment (no weights read).
# kappa_two (far_mode 3): 32-pair steps whose far pairs all lie beyond that many
# lengths take the 2-point rule; 0 = always 3 points.
function calcSegSegForceSurrogateGPU(s::Surrogate, dlnParams, matParams, network;
                                     audit_fraction = 0.01, audit_tol = 1e-3, exact_mode = 0, far_mode = 0,
                                     kappa_two = far_mode == 3 ? 30.0 : 0.0)
    nu = 1 - matParams.μ4π / matParams.μ4πν
    far_mode != 0 || isnan(s.nu) || abs(nu - s.nu) <= 1e-9 ||
        throw(ArgumentError("surrogate trained for nu = $(s.nu), not $nu"))
    numSeg = network.numSeg[1]
    out = zeros(3, 2, numSeg)
    k = Ref(consts(dlnParams, matParams))
    opts = Ref(DDDSurOpts(s.kappa, audit_fraction, audit_tol, exact_mode, far_mode, kappa_two))
    rep = Ref{DDDSurReport}()
    coord, bVec, segIdx, extSeg = network.coord, network.bVec, network.segIdx, network.extSeg
    GC.@preserve coord bVec segIdx extSeg out begin
        rc = ccall((:ddd_surrogate_force_host, libddd), Cint,
            (Ptr{Cvoid}, Ref{DDDConsts}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Int64}, Int64,
             Ptr{Bool}, Int64, Ptr{Float64}, Ref{DDDSurOpts}, Ref{DDDSurReport}),
            s.ptr, k, coord, size(coord, 2), bVec, size(bVec, 2), segIdx, size(segIdx, 1),
            extSeg, numSeg, out, opts, rep)
    end
    surcheck(s, rc)
    return out, rep[]
end

end # module
