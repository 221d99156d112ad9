function P = rtmcProblem(geometry, source, material, obs, ibins, opts)
%RTMCPROBLEM  The rtmc_problem fields (include/rtmc.h) that rtmc_mex reads.
%   P = rtmcProblem(geometry, source, material, obs, ibins) sets up one GPU transport
%   from the structures radiativeTransfer builds: obs and ibins from
%   initializeObservation, material after MaterialClass.prepareSigma.  It restates the
%   set-up of propagateParticleSmallDt.m:3-82 (sub-step, Q rates), initializeParticle.m
%   (point source, radial profile, plane wave) and the boundary list of geometry.bnd.
%   The observation axes ibins are binned; the other axes are range checks on their two
%   edges, as observeTime.m does with vals.
%
%   opts (optional struct): precision 'fp32' (default) or 'fp64', seed (0), pid0 (0),
%   hist_shift (0: plain counts), max_events (0: automatic event cap).
if nargin < 6, opts = struct(); end
d = geometry.dimension;
frames = {'cartesian', 'cylindrical', 'spherical'};
P.d = d;
P.frame = find(strcmp(geometry.frame, frames)) - 1;
P.acoustics = double(material.acoustics);
P.precision = double(isfield(opts, 'precision') && strcmp(opts.precision, 'fp64'));
P.seed = optval(opts, 'seed', 0);
P.pid0 = optval(opts, 'pid0', 0);
P.hist_shift = optval(opts, 'hist_shift', 0);
P.max_events = optval(opts, 'max_events', 0);
P.n_particles = obs.N;

% time grid: obs.t(1) = 0 is never filled; instants 2..Nt are observed
T = mean(diff(obs.t));
P.n_obs = obs.Nt - 1;
mft = material.meanFreeTime(:).';
if isscalar(mft), mft = [mft mft]; end
P.mft = mft;
largeDt = isprop(material, 'timeSteps') && material.timeSteps == 1;
if largeDt
    % exponential flights in continuous time (propagateParticle.m), served on a grid of
    % 2^20 sub-steps per interval, fewer when the run would exceed 2^30 sub-steps
    P.n_sub = 2^20;
    while P.n_sub > 1 && P.n_sub * P.n_obs >= 2^30
        P.n_sub = P.n_sub / 2;
    end
else
    P.n_sub = ceil(T / min(0.01 * min(mft), T));  % propagateParticleSmallDt.m:4-7
end
P.h = T / P.n_sub;

% speeds, conversion probabilities, intrinsic attenuation (propagateParticleSmallDt.m:31-82)
if material.acoustics
    P.v = [material.v material.v];
    P.p2p = 1; P.s2s = 1;
else
    P.v = [material.vp material.vs];
    P.p2p = material.P2P; P.s2s = material.S2S;
end
Q = Inf;
if isprop(material, 'Q') && ~isempty(material.Q), Q = material.Q(:).'; end
if isscalar(Q) || material.acoustics, Q = [Q(1) Q(1)]; end
P.qrate = [0 0];
if ~largeDt && any(isfinite(Q))
    if ~isprop(material, 'Frequency') || isempty(material.Frequency)
        error('A finite quality factor Q needs material.Frequency');
    end
    omega = 2 * pi * material.Frequency(1);
    P.qrate = (omega * P.h ./ Q) .* isfinite(Q);
end

% source (initializeParticle.m)
if ~isfield(source, 'type') || isempty(source.type), source.type = 'point'; end
pos = [0 0 0];
if isfield(source, 'position') && ~isempty(source.position), pos(1:numel(source.position)) = source.position; end
P.src_pos = pos;
P.src_lambda = 0;
if isfield(source, 'lambda'), P.src_lambda = source.lambda; end
P.polarization = double(~material.acoustics && isfield(source, 'polarization') && source.polarization == 'S');
P.src_dir = 0;
P.src_type = 0; P.src_aperture = 0;
P.src_normal = [0 0 1]; P.src_u = [1 0 0]; P.src_v = [0 1 0]; P.src_extent = [0 0];
P.src_radial_cdf = []; P.src_radial_r = [];
switch source.type
    case 'point'
        if isfield(source, 'direction') && ischar(source.direction)
            P.src_dir = find(strcmp(source.direction, {'uniform', 'outgoing', 'upper'})) - 1;
        end
        if isfield(source, 'radial') && ~isempty(source.radial)
            [P.src_radial_cdf, P.src_radial_r] = radialKnots(source.radial, d);
        end
    case 'plane'
        n = source.direction(:).';
        if isscalar(n)
            k = abs(n); n = zeros(1, 3); n(k) = sign(source.direction);
        end
        n = n / norm(n);
        B = null(n);
        P.src_type = 1;
        P.src_normal = n; P.src_u = B(:, 1).'; P.src_v = B(:, 2).';
        ap = 'rectangle';
        if isfield(source, 'aperture') && ~isempty(source.aperture), ap = lower(source.aperture); end
        if strcmp(ap, 'circle')
            P.src_aperture = 1; P.src_extent = [source.extent(1) 0];
        elseif isscalar(source.extent)
            P.src_extent = [source.extent source.extent];
        else
            P.src_extent = source.extent(1:2);
        end
    otherwise
        error('unknown source type %s', source.type);
end

% boundaries: planes dir 1-3, cylinder dir 4 (propagateParticleSmallDt.m:146-580)
P.bnd_dir = []; P.bnd_val = []; P.bnd_absorb = [];
if ~largeDt && isfield(geometry, 'bnd')
    for b = 1:numel(geometry.bnd)
        P.bnd_dir(b) = geometry.bnd(b).dir;
        P.bnd_val(b) = geometry.bnd(b).val;
        P.bnd_absorb(b) = double(isfield(geometry.bnd(b), 'type') && strcmp(geometry.bnd(b).type, 'absorbing'));
    end
end
if ~material.acoustics && any(~P.bnd_absorb)
    out = MaterialClass.Zoeppritz(material);
    P.zoe_rpp = out.E_Rpp(:).';
    P.zoe_rsvsv = out.E_Rsvsv(:).';
end

% observation axes X, Y, Z, PSI: ibins binned (column-major strides), the others checked
% against their range; then time and mode
n = [obs.Nx obs.Ny obs.Nz obs.Npsi];
P.axis_mode = ones(1, 4);
if d == 2, P.axis_mode(3) = 0; end
P.axis_mode(ibins) = 2;
P.axis_stride = zeros(1, 4);
P.axis_stride(ibins(1)) = 1;
P.axis_stride(ibins(2)) = n(ibins(1));
P.time_stride = n(ibins(1)) * n(ibins(2));
P.mode_stride = P.time_stride * obs.Nt;
P.hist_len = P.mode_stride * (1 + ~material.acoustics);
end

function v = optval(s, name, dflt)
v = dflt;
if isfield(s, name) && ~isempty(s.(name)), v = s.(name); end
end

function [c, r] = radialKnots(f, d)
% knots of the radial inverse CDF of initializeParticle.m:175-203: pdf ~ r^(d-1) f(r) on
% 10000 points of [0, Rmax], cumulative sum pinned to 0 and 1, flat stretches dropped
Rmax = f.GridVectors{1}(end);
x = linspace(0, Rmax, 10000);
w = (x .^ (d - 1)) .* f(x);
cdf = cumsum(w / trapz(x, w)) * mean(diff(x));
cdf(1) = 0; cdf(end) = 1;
i = find(diff(cdf) > 0);
i = unique([i i + 1]);
[c, first] = unique(sort(cdf(i)));
xs = sort(x(i));
r = xs(first);
end
