% NUFFT_3D  Drop-in @nufft_3d class backed by libnufft3d.so (GB300, sm_103a).
%
%   obj = nufft_3d(om, N, 'J', 6, 'u', 2, 'radial', 1, ...)
%   k   = obj.fNUFT(x);        x [N1 N2 N3 nc]  -> k [M nc]
%   x   = obj.aNUFT(k);        k [M nc]         -> x [N1 N2 N3 nc]
%   im  = obj.iNUFT(raw, maxit, damp, W, constraint, lambda);
%   damp = obj.discrep(data, stddev);
%   k   = obj * x;  x = obj' * k   (mtimes / ctranspose)
%
% Same constructor name/value pairs, read-only properties and method names as
% the reference class (nufft_3d.m:26-43, 54-251).  The sparse matrix H is not
% formed: the plan (sorted samples, deapodization U, density d) lives on the
% GPU inside the library and is released by delete().  Only gpu=1 (single
% precision GPU) is built; other values error in the library.
classdef nufft_3d < handle

    properties (SetAccess = private)
        J(1,1) double         = 4   % kernel width
        u(1,1) double         = 2   % oversampling factor
        N(1,3) double = zeros(1,3)  % image dimensions
        alpha(1,1) double     = 0   % Kaiser-Bessel alpha (0 = Beatty)
        radial(1,1) logical   = 1   % radial (1) or separable (0) kernel
        gpu(1,1) double       = 1   % 1 = libnufft3d on the GPU
        K(1,3) double = zeros(1,3)  % oversampled dimensions
        U                           % deapodization [N1 N2 N3] (single)
        d                           % density weights [M 1] (single)
        nnz(1,1) double       = 0   % samples within bounds
    end

    properties (Access = private, Hidden = true)
        plan = uint64(0)            % libnufft3d plan handle
        M(1,1) double = 0           % number of samples
        adjoint(1,1) logical = false % obj' (ctranspose): * applies aNUFT
        owner = []                  % the object whose plan a transposed view borrows
    end

    methods
        function obj = nufft_3d(om, N, varargin)
            if nargin == 0
                return;
            end
            if ~isnumeric(om) || ~isreal(om) || size(om,1) ~= 3 || isempty(om)
                error('om must be a real array with leading dimension of 3');
            end
            om = reshape(double(om), 3, []);
            if nargin < 2 || isempty(N)
                N = 2 * ceil(max(abs(om), [], 2));
                warning('N argument not supplied - using [%i %i %i]', N);
            end
            if mod(numel(varargin), 2)
                error('''varargin'' must be supplied in string/value pairs');
            end
            opts = struct();
            for i = 1:2:numel(varargin)
                name = varargin{i};
                if ~ischar(name)
                    error('''varargin'' must be supplied in string/value pairs');
                end
                switch name
                    case {'J', 'u', 'alpha', 'radial', 'gpu', 'density_iters'}
                        opts.(name) = double(varargin{i+1});
                    case 'd'
                        opts.d = single(varargin{i+1}(:));
                    otherwise
                        error('unknown option ''%s''', name);
                end
            end
            obj.plan = nufft3d_mex('create', om, double(N(:))', opts);
            s = nufft3d_mex('info', obj.plan);
            obj.J = s.J; obj.u = s.u; obj.alpha = s.alpha; obj.radial = s.radial ~= 0;
            obj.N = s.N; obj.K = s.K; obj.nnz = s.nnz; obj.M = s.M;
            if isfield(opts, 'gpu'), obj.gpu = opts.gpu; end
            obj.U = nufft3d_mex('deap', obj.plan);
            obj.d = nufft3d_mex('getd', obj.plan);
        end

        function delete(obj)
            % a transposed view borrows its owner's plan
            if obj.plan ~= 0 && isempty(obj.owner)
                nufft3d_mex('destroy', obj.plan);
            end
            obj.plan = uint64(0);
        end
    end

    methods (Access = private)
        function [nc, nr, ny] = raw_shape(obj, raw)
            % leading dimension(s) [M] or [nr ny] (iNUFT.m:26-39)
            nr = []; ny = [];
            if size(raw, 1) == obj.M
                nc = size(raw, 2);
                extra = numel(raw) / (obj.M * nc);
            else
                if size(raw, 1) * size(raw, 2) ~= obj.M
                    error('raw data leading dimension(s) must be length %i (not %ix%i)', ...
                          obj.M, size(raw, 1), size(raw, 2));
                end
                nr = size(raw, 1); ny = size(raw, 2); nc = size(raw, 3);
                extra = numel(raw) / (obj.M * nc);
            end
            if extra ~= 1
                error('raw data size [%s] seems to have too many dimensions', num2str(size(raw)));
            end
        end
    end
end
