set output "hist_cfg1_MOTIF00027.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-34.3549:10.8915]
set yrange [0:1822]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00027.dat" using 1:2 title 'MOTIF00027 (cfg1)' with boxes
