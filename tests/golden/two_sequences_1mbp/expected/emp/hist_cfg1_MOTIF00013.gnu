set output "hist_cfg1_MOTIF00013.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-24.9394:8.86303]
set yrange [0:1527]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00013.dat" using 1:2 title 'MOTIF00013 (cfg1)' with boxes
