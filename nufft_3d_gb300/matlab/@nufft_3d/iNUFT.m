% im = obj.iNUFT(raw, maxit, damp, W, constraint, lambda, solver, tol)
%
%  raw        complex [M nc] or [nr ny nc]
%  maxit      iterations (0 or 1: regridding aNUFT(d .* raw)); default 20
%  damp       Tikhonov damping; default 0
%  W          [] or a scalar, [ny] or [nr*ny] nonnegative weights (times d)
%  constraint '' (default) or 'phase-constraint' (with lambda); the
%             reference's other experimental constraints ('compressed-sensing',
%             'parallel-imaging-sake', 'parallel-imaging-pruno') need its
%             external 'parallel' package and raise an error here
%  lambda     regularisation parameter of the constraint
%  solver     'minres' (default, as the reference) or 'cg'; tol default 1e-4
%             (these two trailing arguments have no counterpart in the
%             reference, whose argument order up to lambda is kept)
%
% Each coil is solved as its own system (A'WA + damp^2 I) x = A'W raw on the
% GPU (iNUFT.m:2-138, 140-168, 224-227 of the reference).
function [im, iters] = iNUFT(obj, raw, maxit, damp, W, constraint, lambda, solver, tol)
if nargin < 3 || isempty(maxit), maxit = 20; end
if nargin < 4 || isempty(damp), damp = 0; end
if nargin < 5, W = []; end
if nargin < 6, constraint = ''; end
if nargin < 7, lambda = []; end
if nargin < 8 || isempty(solver), solver = 'minres'; end
if nargin < 9 || isempty(tol), tol = 1e-4; end
validateattributes(maxit, {'numeric'}, {'scalar', 'finite', 'integer', 'nonnegative'}, '', 'maxit');
validateattributes(damp, {'numeric'}, {'scalar', 'finite', 'nonnegative'}, '', 'damp');
[nc, nr, ny] = obj.raw_shape(raw);
Wv = [];
if numel(W) > 1
    if maxit <= 1
        warning('weighting is only effective when maxit>1');
    end
    W = double(W(:));
    if numel(W) ~= obj.M
        if isempty(ny), ny = numel(W); nr = obj.M / ny; end
        if mod(nr, 1) || nr * ny ~= obj.M
            error('W must be a vector of length ny or ny*nr');
        end
        W = repmat(reshape(W, 1, ny), nr, 1);
    end
    if any(~isfinite(W(:))) || any(W(:) < 0)
        error('W must be finite and nonnegative');
    end
    Wv = single(W(:));
end
phase = false;
if ~isempty(constraint)
    if maxit <= 1
        warning('phase constraint is only effective when maxit>1');
    else
        switch constraint
            case 'phase-constraint'
                phase = true;
            case {'compressed-sensing', 'parallel-imaging-sake', 'parallel-imaging-pruno'}
                error('constraint ''%s'' is not implemented (it needs the external ''parallel'' package)', ...
                      constraint);
            otherwise
                error('unknown constraint');
        end
        if isempty(lambda)
            error('lambda must be supplied with %s', constraint);
        end
        validateattributes(lambda, {'numeric'}, {'scalar', 'finite', 'nonnegative'}, '', 'lambda');
    end
end
raw = single(reshape(raw, obj.M, nc));
if isreal(raw), raw = complex(raw); end
if phase
    [im, iters] = nufft3d_mex('inverse_phase', obj.plan, raw, double(maxit), double(damp), double(lambda), ...
                              Wv, double(tol));
else
    [im, iters] = nufft3d_mex('inverse', obj.plan, raw, double(maxit), double(damp), Wv, solver, double(tol));
end
